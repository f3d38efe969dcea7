// Shared declarations of the GB300 assembly kernels: the device-resident plan,
// device term descriptors, error plumbing and small device helpers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/fem_g_gb300.h"

namespace femg {

void setLastError(const std::string &msg);
void countLaunch(int n = 1);

// Brackets one kernel launch with CUDA events on its stream while the kernel
// timer (fg_profile_enable) is on; a no-op otherwise.
// while suspended (stream capture), this thread's ProfScopes record nothing
void profSuspend(bool on);
// whether the kernel timer is on (fg_profile_enable)
bool profEnabled();

class ProfScope {
 public:
  ProfScope(const char *name, cudaStream_t s);
  ~ProfScope();

 private:
  const char *name_;
  cudaStream_t s_;
  cudaEvent_t a_ = nullptr, b_ = nullptr;
};

#define FG_CUDA(call)                                                                          \
  do {                                                                                         \
    cudaError_t _e = (call);                                                                   \
    if (_e != cudaSuccess) {                                                                   \
      ::femg::setLastError(std::string(#call) + ": " + cudaGetErrorString(_e));              \
      return FG_ERR_CUDA;                                                                      \
    }                                                                                          \
  } while (0)

// Dynamic shared memory above 48 KB has to be allowed per kernel on every
// device that runs it; a SmemAllowance remembers, per device ordinal, the
// largest size already allowed for one kernel (races only repeat the call).
constexpr int kSmemMaxDevices = 64;
struct SmemAllowance {
  size_t bytes[kSmemMaxDevices] = {};
};
template <typename K>
inline cudaError_t allowSmem(K kern, size_t smem, SmemAllowance &a) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < kSmemMaxDevices && smem <= a.bytes[dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess && dev >= 0 && dev < kSmemMaxDevices) a.bytes[dev] = smem;
  return e;
}

constexpr int kMaxDofs = 64;         // element DOFs (basis x multiplicity) handled on device
constexpr int kMaxNodes = 10;        // geometric nodes per element
constexpr int kMaxTerms = 6;
constexpr int kOutChunks = 8;        // row ranges of the gather for overlapped host copies
constexpr uint16_t kSlotFixed = 0xFFFF;   // column is a fixed DOF (Dirichlet lifting)
constexpr uint16_t kSlotIgnore = 0xFFFE;  // column does not assemble (undefined type)

// Device copy of an fg_expr with device array pointers and a precomputed class
enum ExprClass { kExprConst = 0, kExprElem = 1, kExprPoint = 2 };
struct DevExpr {
  int32_t n_code;
  int32_t cls;
  double2 cval;  // value when cls == kExprConst
  fg_instr code[FG_EXPR_MAX_CODE];
  const double2 *arr[FG_EXPR_MAX_ARRAYS];
};

struct DevJacMod {
  int32_t kind, axis, exponent, pad_;
  double rmin, rmax, center[3];
};

struct DevTerm {
  int32_t kind;
  int32_t dt;
  double2 factor;  // module factor: 1, -omega^2 (dt2) or -i omega (dt1)
  DevExpr coef, coef2;
  int32_t mod;     // index of the term's Jacobian modificator in DevTerms::mods
  int32_t pad_;
};

struct DevTerms {
  int32_t n;
  int32_t complexKe;   // element matrices need an imaginary part
  int32_t hasSource;
  int32_t hasElastic;
  int32_t nMod;        // distinct Jacobian modificators of the terms (>= 1; FG_JACMOD_NONE counts)
  int32_t hasJacMod;   // some term has a modificator other than FG_JACMOD_NONE
  int32_t tensorTerm;  // index of the FG_TERM_GRAD_GRAD_TENSOR term (at most one), -1 when none
  int32_t tensorMassTerm;  // index of the FG_TERM_MASS_TENSOR term (HCurl; at most one), -1 when none
  int32_t tensorPoint; // some entry of those tensors depends on the point
  int32_t pad_;
  DevTerm t[kMaxTerms];
  DevJacMod mods[kMaxTerms];
  DevExpr tensor[6];   // entries (00, 11, 22, 01, 02, 12) of the grad-grad (curl-curl) term's symmetric tensor
  DevExpr tensorMass[6];  // the same for the mass term's tensor
  // terms with non-symmetric element matrices (scalar H1, FP64 paths)
  int32_t nonSym;          // a full-tensor, advection or vector term is present
  int32_t tensorFullTerm;  // index of the FG_TERM_GRAD_GRAD_TENSOR_FULL term, -1 when none
  int32_t advectTerm;      // index of the FG_TERM_ADVECTION term, -1 when none
  int32_t vecGradTerm;     // index of the FG_TERM_VECTOR_GRAD_TEST term, -1 when none
  int32_t srcGradTerm;     // index of the FG_TERM_SOURCE_GRAD term, -1 when none
  int32_t pad2_;
  DevExpr tensorFull[9];   // its D, row-major
  DevExpr advect[3];       // the advection vector b
  DevExpr vecGrad[3];      // b of integral(b dof(u), grad(tf(u)))
  DevExpr srcGrad[3];      // f of integral(f, grad(tf(u)))
};

// Device-resident data of one element bucket
struct PlanDev {
  int32_t dim, nn, nq, nb, mult, n, nOrient, affine;
  int32_t p1geom;         // first-order simplex geometry with the standard node order
  int32_t form;           // FG_FORM_0 (H1) or FG_FORM_1 (HCurl: vector values, curls)
  int64_t E, nNodes;
  uint64_t nRows, nnz, nFixed;
  const double *xyz;      // [nNodes][3]
  const int32_t *enodes;  // [E][nn]
  const double *w;        // [nq]
  const double *geoVal;   // [nq][nn]
  const double *geoGrad;  // [nq][nn][3]
  const double *bval;     // [nOrient][nq][nb] (FG_FORM_1: [nOrient][nq][nb][3] vector values)
  const double *bgrad;    // [nOrient][nq][nb][3] gradients (FG_FORM_1: curls)
  const int32_t *orient;  // [E] or null
  const uint32_t *edof;   // [E][n]: row/column index, or fixed index for fixed DOFs
  const uint8_t *etype;   // [E][n]: FG_AT_*
  const uint64_t *ai;     // [nRows+1]
  const uint64_t *rowPtr; // [nRows+1] into rowElem
  const uint32_t *rowElem;// (e << 6) | i : element and local test index
  const uint4 *visit;      // per visited row: row, CSR start, element-list start, len | count << 16
  const uint32_t *visitElem;// element lists in visiting order
  const void *slot;       // [E][n][slotLd] uint8 or uint16 position in the row
  int32_t slotBytes;
  int32_t slotLd;         // slot row stride (entries)
  int32_t maxRowLen;
  int32_t plainSlots;     // 1: no element row has two columns in one slot (plain shared adds are race-free)
  int *jmErr;             // set by the FP64 element kernels: an integration point outside a shell
  const double2 *lscale;  // [E][n] linked DOF coefficient (1 for other DOFs), or null without linked DOFs
  // The columns: the unknown field's DOFs. A plan of one field has them equal
  // to the rows (nc = n, the U tables alias the ones above); a two-field plan
  // (fg_plan_create_coupled) has the test field's DOFs as rows and the
  // unknown field's as columns, element matrices [E][n][nc].
  int32_t coupled;        // 1: two-field plan
  int32_t nc, nbU, nOrientU;
  const double *bvalU;    // [nOrientU][nq][nbU]
  const double *bgradU;   // [nOrientU][nq][nbU][3]
  const int32_t *orientU; // [E] or null
  const uint32_t *edofU;  // [E][nc]: column index, or fixed index for fixed DOFs
  const uint8_t *etypeU;  // [E][nc]: FG_AT_*
};

}  // namespace femg

struct fg_plan {
  femg::PlanDev d;
  // host copies needed by later calls
  std::vector<uint64_t> hAi;
  int64_t E = 0;
  // row ranges of the gather's visiting order ([k] .. [k + 1]), copied out
  // one by one when the CSR values go to the host
  std::vector<uint64_t> outChunkRow;
  const uint4 *visitRanged = nullptr;         // the visit tables in range-major order
  const uint32_t *visitElemRanged = nullptr;
  cudaStream_t copyStream = nullptr;
  std::vector<cudaEvent_t> copyEvents;
  // owned device allocations
  std::vector<void *> allocs;
  // scratch (grown on demand)
  double *ke = nullptr;
  size_t keBytes = 0;
  double *be = nullptr;
  size_t beBytes = 0;
  double *dirichlet = nullptr;
  size_t dirichletBytes = 0;
  double *values = nullptr;  // device CSR values when the caller passes host memory
  size_t valuesBytes = 0;
  double *rhs = nullptr;
  size_t rhsBytes = 0;
  std::vector<void *> termArrays;   // device copies of per-element coefficient arrays (per call)
  std::unordered_map<void *, size_t> arrayBytes;  // allocated size of each coefficient array
  std::vector<void *> boundArrays;  // ... of the terms bound by fg_plan_bind_terms
  femg::DevTerms bound;
  femg::DevTerms *boundDev = nullptr;  // device copy of the bound terms
  femg::DevTerms *termsDev = nullptr;  // device copy of the last per-call terms
  bool hasBound = false;
  bool fixedColumns = false;  // a two-field plan with fixed unknown DOFs (lifting into the test rows)
  // mixed-precision state (reference tensors per orientation), see assemble_mixed.cu
  void *mixed = nullptr;
  // multi-frequency state (term groups, element matrices), see multi_freq.cu
  void *multi = nullptr;
  // FP64 factorization state (reference tensors, tiles), see assemble_fp64f.cu
  void *fp64f = nullptr;
  int fp64Method = 0;  // FG_FP64_* (FG_FP64_QUADRATURE)
  int accumulate = 0;  // add into device outputs instead of overwriting them (fg_plan_set_accumulate)
  // fused mixed path (contraction and reduction in one kernel), see fused.cu
  void *fused = nullptr;
  int mixedFused = 0;  // fg_plan_set_mixed_fused (off by default)
  int *jmErrHost = nullptr;  // pinned copy of d.jmErr
};

namespace femg {

// grow-only device scratch
int ensureDevice(void **ptr, size_t *cap, size_t bytes);
// upload a term list (copies per-element arrays)
int uploadTerms(fg_plan *plan, const fg_term_desc *terms, int32_t nTerms, double frequency, DevTerms *out,
                std::vector<void *> &arrays);
// terms of a call: uploaded now, or the bound ones when terms == NULL
int resolveTerms(fg_plan *plan, const fg_term_desc *terms, int32_t nTerms, double frequency, DevTerms *out,
                 const DevTerms **dev, cudaStream_t s);
// multiprocessor count of the current device (cached)
int smCount();
// copy the Dirichlet values; return device pointer (or null)
int uploadDirichlet(fg_plan *plan, const double *dirichlet, const double **out, cudaStream_t s);
bool isDevicePointer(const void *p);
// Layout of the element matrices the reduction reads: row-major [n][n]
// (FP64 kernels, scalar and HCurl fields) or 3x3 component blocks
// [a*3+b][nb][nb] (compound fields on the tensor-core path). ld = entries per
// component (imaginary part at +ld, next element at +ncomp*ld). A packed
// upper triangle for the symmetric scalar case halved the contraction's
// output but made the reduction's reads of the lower half scattered: the
// 384,000-tet order-3 step went from 0.854 to 0.877 ms, so it is not used.
enum { kKeFull = 0, kKeBlocks3 = 1 };
struct KeLayout {
  int32_t kind, ld;
};
inline KeLayout keFull(int n) { return KeLayout{kKeFull, n * n}; }
// full layout of a two-field plan: n rows of nc entries
inline KeLayout keRect(int n, int nc) { return KeLayout{kKeFull, n * nc}; }
// offset of entry (ii, jj); n: entries per row in the full layout (the
// columns nc), the basis count times 3 in the compound one
__device__ __forceinline__ int keOffset(const KeLayout &lay, int n, int ii, int jj) {
  if (lay.kind == kKeFull) return ii * n + jj;
  const int nb = n / 3, i = ii / 3, a = ii - 3 * i, j = jj / 3, b = jj - 3 * j;
  return ((a * 3 + b) * nb + i) * nb + j;
}
// FG_ERR_UNSUPPORTED (with the message set) when a two-field plan would lift
// fixed unknown DOFs into `rhs` through a block of n != nc: the reference's
// addValuesDC reads values[j * nc + i] there, outside the element matrix
int coupledLiftCheck(const fg_plan *plan, const double *rhs);
// gather of element matrices/vectors into CSR values and RHS
int launchGather(fg_plan *plan, const double *ke, int keComplex, int keIsFloat, KeLayout lay, const double *be,
                 const double *dirichletDev, double *values, double *rhs, cudaStream_t s);
// outputs: device pointers used in place, host pointers staged through the plan
struct Outputs {
  double *values = nullptr, *rhs = nullptr;
  bool hostValues = false, hostRhs = false;
  bool valuesCopied = false;  // the host copy of the values is already queued (range by range)
};
int prepareOutputs(fg_plan *plan, double *csr_values, double *rhs, Outputs *o);
int finishOutputs(fg_plan *plan, const Outputs &o, double *csr_values, double *rhs, cudaStream_t s);
// The CSR reduction into the outputs: with host values, range by range, each
// range's slice copied to the host on a second stream while the next reduces
int gatherToOutputs(fg_plan *plan, const double *ke, int keComplex, int keIsFloat, KeLayout lay, const double *be,
                    const double *dirichletDev, Outputs &o, double *csr_values, cudaStream_t s);
// Fused mixed path: whether a call of these terms runs fused (builds the
// block records on first use), the launch, and its wait-timeout report
bool fusedApplies(fg_plan *plan, const DevTerms &dt);
int launchFused(fg_plan *plan, const DevTerms &dt, const DevTerms *dterms, const double2 *be, double2 *values, double2 *rhs,
                cudaStream_t s);
int fusedTimeout(fg_plan *plan, bool wait);
// Factor rows [hi | lo] (16 floats) in element order for the fused kernel
int launchFactorsCompact(const PlanDev &p, const DevTerms *dterms, bool tensor, float *A16, cudaStream_t s);
// B' image of orientation o in the shared-memory core-matrix layout (Npad x K'
// floats; compact: K' = 2 kp [B_hi ; B_lo], else 3 kp [B_hi ; B_hi ; B_lo])
void buildB(const PlanDev &p, const std::vector<double> &w, const std::vector<double> &bval, const std::vector<double> &bgrad,
            int o, int Npad, int kp, std::vector<float> &img, bool compact);
// FP64 element kernel (also used as the reference for the mixed error report)
int launchElementFp64(fg_plan *plan, const DevTerms &terms, const DevTerms *dterms, double *ke, double *be, cudaStream_t s);
// One plan of a batched gather launch
struct GatherJob {
  PlanDev p;
  const void *ke;  // element matrices (float or double, one layout per launch)
  const double2 *be, *uD;
  double2 *values, *rhs;
  KeLayout lay;
  int64_t blockStart, nBlocks;
};
struct GatherShape {
  int L = 0, J = 3, wpb = 0, rowsPerBlock = 0;  // lanes per row, columns per lane
  size_t smem = 0;
  bool ok = false;
  bool v4 = false;  // k_gather_batch_v4: L = n / 4 lanes, 4 columns each by vector loads
};
// L, wpb <= 0: the defaults of the single-plan gather
GatherShape gatherShape(int n, int maxRowLen, int kcplx, int keIsFloat, int L, int wpb);
// the vector-load shape (real FP32 element matrices, n a multiple of 4 up to 32)
GatherShape gatherShapeV4(int n, int maxRowLen, int wpb);
int launchGatherBatch(const GatherJob *jobsDev, int nJobs, int64_t blocks, int slotBytes, int kcplx, int keIsFloat,
                      const GatherShape &g, cudaStream_t s);

// One problem (element bucket) of a tensor-core contraction launch
struct GemmProblem {
  const float *A;       // [rows][K3] split factor rows
  const float *B;       // [nOrient][Npad * K3] core-matrix images
  const int32_t *perm;  // rank -> element
  float *ke;            // [E][rowsPerElem][ld]
  int Npad, nn2, rowsPerElem, K3;
  int mmaN;             // N of one MMA instruction (16..256, multiple of 16)
  int ld;               // element-matrix row stride (floats): nn2, or nn2 padded to a multiple of 8
};

// One plan of a batched factor-row launch (mixed path)
struct FactorJob {
  PlanDev p;
  const DevTerms *terms;
  const int32_t *rankOf;
  float *A;
  int32_t ncomp, rowsPerElem, rowOff, kind;  // kind: 0 scalar H1, 1 Tensor4 compound, 2 HCurl, 3 scalar H1 with a tensor term
  int64_t elemStart;
};

// FP64 element matrices by factorization (assemble_fp64f.cu): affine elements,
// element-constant bilinear coefficients, one-component fields
bool factoredFp64Applies(const fg_plan *plan, const DevTerms &terms);
int launchFactoredFp64(fg_plan *plan, const DevTerms &terms, const DevTerms *dterms, double *ke, cudaStream_t s);

// mixed path pieces shared with the multi-frequency path (assemble_mixed.cu)
int prepareMixed(fg_plan *plan, int ncomp, int groups);
int launchMixedElement(fg_plan *plan, const DevTerms *const *dterms, int groups, uint32_t tensorMask, cudaStream_t s);
int launchRhsFp64(fg_plan *plan, const DevTerms *dterms, double *be, cudaStream_t s);
float *mixedKe(fg_plan *plan, KeLayout *lay);
int mixedCheckTimeout(fg_plan *plan, bool wait);
int mixedRecordError(fg_plan *plan, cudaStream_t s);
// ... and with the batch (batch.cu)
int launchFactorsBatch(const FactorJob *jobsDev, int nJobs, int64_t total, cudaStream_t s);
FactorJob mixedFactorJob(fg_plan *plan, const DevTerms *dterms, bool tensor, int64_t elemStart);
std::vector<int4> mixedTiles(fg_plan *plan, int prob, int rowsPerElem);
// contraction CTAs per SM (1 or 2) and the dynamic shared memory that pins it
int gemmCtasPerSm(int Npad, int k3);
size_t gemmSmem(int Npad, int k3, int ctasPerSm = 1);
std::vector<int32_t> partitionTiles(const std::vector<double> &cost, int nCta);
// next: the tile counter of a dynamic schedule (chunks of `chunk` tiles out
// of nTiles; zeroed on the stream before the launch), or null for the
// static ranges of ctaStartDev
int launchContract(const void *probsDev, const int4 *tilesDev, const int32_t *ctaStartDev, int nCta, int *err, int maxK3,
                   size_t smem, cudaStream_t s, int tmemCols = 512, const void *aMap = nullptr, int *next = nullptr,
                   int nTiles = 0, int chunk = 0);
GemmProblem mixedGemmProblem(fg_plan *plan);

// ------------------------------------------------------------- device helpers

__host__ __device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

__device__ inline double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// Exact FP32 -> FP64 widening with integer operations. The F2F instruction
// runs on the FP64 pipe, which is narrow on GB300; the bit manipulation runs
// on the integer pipes. Handles zeros, subnormals, infinities and NaNs.
__device__ inline double widen(float x) {
  const uint32_t b = __float_as_uint(x);
  const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
  const uint32_t ex = (b >> 23) & 0xFFu;
  uint32_t man = b & 0x7FFFFFu;
  uint64_t bits;
  if (ex == 0xFFu) {
    bits = sign | (0x7FFull << 52) | ((uint64_t)man << 29);
  } else if (ex != 0) {
    bits = sign | ((uint64_t)(ex + 896u) << 52) | ((uint64_t)man << 29);  // 1023 - 127 = 896
  } else if (man == 0) {
    bits = sign;
  } else {
    // subnormal: value = man * 2^-149; normalise the leading one to bit 23
    const int lz = __clz(man) - 8;  // shift that brings the leading one to bit 23
    man = (man << lz) & 0x7FFFFFu;
    bits = sign | ((uint64_t)(897 - lz) << 52) | ((uint64_t)man << 29);
  }
  return __longlong_as_double((long long)bits);
}
__device__ inline double widen(double x) { return x; }

// Complex elementary functions of the coefficient language (the scalar
// operators of src/function/scalarUnaryOperators.h on std::complex<double>),
// written from their definitions with CUDA's real math functions, principal
// branches as in C99 Annex G / std::complex:
//   exp z = e^x (cos y, sin y); ln z = (ln|z|, arg z); sqrt by the half-angle
//   form with the sign of y; sin, cos, sinh, cosh by the addition theorems;
//   tan = sin / cos, tanh = sinh / cosh; the inverse functions through ln and
//   sqrt: asin z = -i ln(i z + sqrt(1 - z^2)), acos z = pi/2 - asin z,
//   atan z = (i/2) (ln(1 - i z) - ln(1 + i z)), asinh z = ln(z + sqrt(z^2 + 1)),
//   acosh z = ln(z + sqrt(z + 1) sqrt(z - 1)), atanh z = (ln(1 + z) - ln(1 - z)) / 2;
//   z^p for a real power p: x^p when z is real and positive, else
//   |z|^p (cos p arg z, sin p arg z), as std::pow(complex, real) does.
__device__ inline double2 cexpD(double2 z) {
  double s, c;
  sincos(z.y, &s, &c);
  const double e = exp(z.x);
  return make_double2(e * c, e * s);
}
__device__ inline double2 clnD(double2 z) { return make_double2(log(hypot(z.x, z.y)), atan2(z.y, z.x)); }
__device__ inline double2 csqrtD(double2 z) {
  if (z.x == 0.0 && z.y == 0.0) return make_double2(0.0, z.y);
  const double t = sqrt(0.5 * (hypot(z.x, z.y) + fabs(z.x)));
  if (z.x >= 0.0) return make_double2(t, z.y / (2.0 * t));
  return make_double2(fabs(z.y) / (2.0 * t), copysign(t, z.y));
}
__device__ inline double2 csinD(double2 z) {
  double s, c;
  sincos(z.x, &s, &c);
  return make_double2(s * cosh(z.y), c * sinh(z.y));
}
__device__ inline double2 ccosD(double2 z) {
  double s, c;
  sincos(z.x, &s, &c);
  return make_double2(c * cosh(z.y), -s * sinh(z.y));
}
__device__ inline double2 csinhD(double2 z) {
  double s, c;
  sincos(z.y, &s, &c);
  return make_double2(sinh(z.x) * c, cosh(z.x) * s);
}
__device__ inline double2 ccoshD(double2 z) {
  double s, c;
  sincos(z.y, &s, &c);
  return make_double2(cosh(z.x) * c, sinh(z.x) * s);
}
__device__ inline double2 cpowRealD(double2 z, double p) {
  if (z.y == 0.0 && z.x > 0.0) return make_double2(pow(z.x, p), 0.0);
  const double r = pow(hypot(z.x, z.y), p), th = p * atan2(z.y, z.x);
  double s, c;
  sincos(th, &s, &c);
  return make_double2(r * c, r * s);
}
__device__ inline double2 cUnary(int op, int arg, double2 z) {
  const double2 one = make_double2(1.0, 0.0);
  const double2 iz = make_double2(-z.y, z.x);  // i z
  switch (op) {
    case FG_OP_SQRT: return csqrtD(z);
    case FG_OP_EXP: return cexpD(z);
    case FG_OP_LN: return clnD(z);
    case FG_OP_LOG10: {
      const double2 l = clnD(z);
      const double k = 1.0 / log(10.0);
      return make_double2(l.x * k, l.y * k);
    }
    case FG_OP_POW: {
      if (arg == 1) return z;
      if (arg == 2) return cmul(z, z);
      if (arg == 3) return cmul(cmul(z, z), z);
      if (arg == 4) {
        const double2 z2 = cmul(z, z);
        return cmul(z2, z2);
      }
      return cpowRealD(z, (double)arg);
    }
    case FG_OP_CBRT: return cpowRealD(z, 1.0 / 3.0);
    case FG_OP_SIN: return csinD(z);
    case FG_OP_COS: return ccosD(z);
    case FG_OP_TAN: return cdiv(csinD(z), ccosD(z));
    case FG_OP_SINH: return csinhD(z);
    case FG_OP_COSH: return ccoshD(z);
    case FG_OP_TANH: return cdiv(csinhD(z), ccoshD(z));
    case FG_OP_ASIN: {
      const double2 w = clnD(cadd(iz, csqrtD(make_double2(1.0 - (z.x * z.x - z.y * z.y), -2.0 * z.x * z.y))));
      return make_double2(w.y, -w.x);  // -i w
    }
    case FG_OP_ACOS: {
      const double2 a = cUnary(FG_OP_ASIN, 0, z);
      return make_double2(1.5707963267948966 - a.x, -a.y);
    }
    case FG_OP_ATAN: {
      const double2 a = clnD(make_double2(1.0 - iz.x, -iz.y)), b = clnD(cadd(one, iz));
      const double2 d = make_double2(a.x - b.x, a.y - b.y);
      return make_double2(-0.5 * d.y, 0.5 * d.x);  // (i / 2) d
    }
    case FG_OP_ASINH: return clnD(cadd(z, csqrtD(make_double2(z.x * z.x - z.y * z.y + 1.0, 2.0 * z.x * z.y))));
    case FG_OP_ACOSH:
      return clnD(cadd(z, cmul(csqrtD(make_double2(z.x + 1.0, z.y)), csqrtD(make_double2(z.x - 1.0, z.y)))));
    case FG_OP_ATANH: {
      const double2 a = clnD(make_double2(1.0 + z.x, z.y)), b = clnD(make_double2(1.0 - z.x, -z.y));
      return make_double2(0.5 * (a.x - b.x), 0.5 * (a.y - b.y));
    }
    case FG_OP_ABS: return make_double2(hypot(z.x, z.y), 0.0);
    case FG_OP_CONJ: return make_double2(z.x, -z.y);
    case FG_OP_REAL: return make_double2(z.x, 0.0);
    case FG_OP_IMAG: return make_double2(z.y, 0.0);
  }
  return z;
}

// Evaluate a coefficient expression at element e and physical point x; phi:
// the scalar basis values at the point (nb of them) for field nodes, null
// where the expression is evaluated once per element (field nodes make an
// expression point-dependent, which those paths refuse); q and nq: the
// point's index in the rule and the rule's size, for point tables
__device__ inline double2 evalExpr(const DevExpr &ex, int64_t e, const double *x, const double *phi = nullptr, int nb = 0,
                                   int q = 0, int nq = 1) {
  if (ex.cls == kExprConst) return ex.cval;
  double2 st[16];
  int sp = 0;
  for (int k = 0; k < ex.n_code; ++k) {
    const fg_instr in = ex.code[k];
    switch (in.op) {
      case FG_OP_CONST: st[sp++] = make_double2(in.re, in.im); break;
      case FG_OP_X: st[sp++] = make_double2(x[0], 0.0); break;
      case FG_OP_Y: st[sp++] = make_double2(x[1], 0.0); break;
      case FG_OP_Z: st[sp++] = make_double2(x[2], 0.0); break;
      case FG_OP_ELEM: st[sp++] = ex.arr[in.arg][e]; break;
      case FG_OP_POINT: st[sp++] = ex.arr[in.arg][e * nq + q]; break;
      case FG_OP_FIELD: {
        const double2 *u = ex.arr[in.arg] + (size_t)e * nb;
        double2 s = make_double2(0.0, 0.0);
        for (int j = 0; phi && j < nb; ++j) {
          const double2 v = u[j];
          s.x += phi[j] * v.x;
          s.y += phi[j] * v.y;
        }
        st[sp++] = s;
        break;
      }
      case FG_OP_NEG: st[sp - 1] = make_double2(-st[sp - 1].x, -st[sp - 1].y); break;
      case FG_OP_HEAVISIDE: {
        const double r = st[sp - 1].x;
        st[sp - 1] = make_double2(r > 0.0 ? 1.0 : (r < 0.0 ? 0.0 : 0.5), 0.0);
        break;
      }
      case FG_OP_ADD:
      case FG_OP_SUB:
      case FG_OP_MUL:
      case FG_OP_DIV:
      case FG_OP_ATAN2: {
        const double2 b = st[--sp];
        const double2 a = st[sp - 1];
        double2 r;
        if (in.op == FG_OP_ADD) r = cadd(a, b);
        else if (in.op == FG_OP_SUB) r = make_double2(a.x - b.x, a.y - b.y);
        else if (in.op == FG_OP_MUL) r = cmul(a, b);
        else if (in.op == FG_OP_DIV) r = cdiv(a, b);
        else r = make_double2(atan2(a.x, b.x), 0.0);
        st[sp - 1] = r;
        break;
      }
      default: st[sp - 1] = cUnary(in.op, in.arg, st[sp - 1]);
    }
  }
  return st[0];
}

// Coefficient tensor of modificator group g at element e and point x:
// A = c0 I + factor c D, with c0 the summed scalar coefficients of the same
// kind and D the entries (00, 11, 22, 01, 02, 12) of tensor term `term`
// (none when term < 0).
__device__ inline void coefTensor(const DevTerms *terms, int term, const DevExpr *D, int g, int64_t e, const double *x, double2 c0,
                                  double2 *A, const double *phi = nullptr, int nb = 0, int q = 0, int nq = 1) {
  for (int k = 0; k < 6; ++k) A[k] = k < 3 ? c0 : make_double2(0.0, 0.0);
  if (term < 0) return;
  const DevTerm &T = terms->t[term];
  if (T.mod != g) return;
  const double2 fc = cmul(T.factor, evalExpr(T.coef, e, x, phi, nb, q, nq));
  for (int k = 0; k < 6; ++k) A[k] = cadd(A[k], cmul(fc, evalExpr(D[k], e, x, phi, nb, q, nq)));
}
// the grad-grad (diffusion) tensor
__device__ inline void diffusionTensor(const DevTerms *terms, int g, int64_t e, const double *x, double2 cgg, double2 *A,
                                       const double *phi = nullptr, int nb = 0, int q = 0, int nq = 1) {
  coefTensor(terms, terms->tensorTerm, terms->tensor, g, e, x, cgg, A, phi, nb, q, nq);
}
// F(a, b) = sum_rs Q[3a + r] A(r, s) Q[3b + s] for the six pairs (a, b), of
// the real (comp 0) or imaginary (comp 1) part of the symmetric A
__device__ inline void congruence6(const double *Q, const double2 *A6, int comp, double *F) {
  const int sym[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
  const int ab[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  double QA[9];
  for (int a = 0; a < 3; ++a)
    for (int s = 0; s < 3; ++s) {
      double v = 0.0;
      for (int r = 0; r < 3; ++r) v += Q[3 * a + r] * (comp == 0 ? A6[sym[r][s]].x : A6[sym[r][s]].y);
      QA[3 * a + s] = v;
    }
  for (int k = 0; k < 6; ++k) {
    const int a = ab[k][0], b = ab[k][1];
    F[k] = QA[3 * a] * Q[3 * b] + QA[3 * a + 1] * Q[3 * b + 1] + QA[3 * a + 2] * Q[3 * b + 2];
  }
}

// Jacobian at a quadrature point from the geometric nodes, stored column-major
// like gmsh's getJacobians (J[3*c + r] = d x_r / d u_c); 2D elements get the
// unit normal as third column. Returns det J.
__device__ inline double jacobian(int dim, int nn, const double *X /*[nn][3]*/, const double *dN /*[nn][3]*/, double *J) {
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) J[3 * c + r] = 0.0;
  const int nc = dim;
  for (int k = 0; k < nn; ++k)
    for (int c = 0; c < nc; ++c) {
      const double g = dN[3 * k + c];
      J[3 * c + 0] += X[3 * k + 0] * g;
      J[3 * c + 1] += X[3 * k + 1] * g;
      J[3 * c + 2] += X[3 * k + 2] * g;
    }
  if (dim == 2) {
    const double nx = J[1] * J[5] - J[2] * J[4];
    const double ny = J[2] * J[3] - J[0] * J[5];
    const double nz = J[0] * J[4] - J[1] * J[3];
    const double len = sqrt(nx * nx + ny * ny + nz * nz);
    J[6] = nx / len;
    J[7] = ny / len;
    J[8] = nz / len;
  }
  // det of the column-major matrix
  return J[0] * (J[4] * J[8] - J[7] * J[5]) - J[3] * (J[1] * J[8] - J[7] * J[2]) + J[6] * (J[1] * J[5] - J[4] * J[2]);
}

// The same for first-order simplex geometry (N_0 = 1 - sum u, N_k = u_k):
// the Jacobian's columns are edge vectors from node 0; X holds dim + 1 nodes.
__device__ inline double jacobianP1(int dim, const double *X, double *J) {
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) J[3 * c + r] = c < dim ? X[3 * (c + 1) + r] - X[r] : 0.0;
  if (dim == 2) {
    const double nx = J[1] * J[5] - J[2] * J[4];
    const double ny = J[2] * J[3] - J[0] * J[5];
    const double nz = J[0] * J[4] - J[1] * J[3];
    const double len = sqrt(nx * nx + ny * ny + nz * nz);
    J[6] = nx / len;
    J[7] = ny / len;
    J[8] = nz / len;
  }
  return J[0] * (J[4] * J[8] - J[7] * J[5]) - J[3] * (J[1] * J[8] - J[7] * J[2]) + J[6] * (J[1] * J[5] - J[4] * J[2]);
}

// inverse-transpose application data: Kinv[a][r] = (J^-1)[a][r], so that the
// physical gradient is G_r = sum_a Kinv[a][r] * dphi/du_a  (J^-T grad)
__device__ inline void jacobianInverse(const double *J, double det, double *Jinv /*row-major [a][r]*/) {
  // J(r,c) = J[3c + r]
  auto Jm = [&](int r, int c) { return J[3 * c + r]; };
  const double id = 1.0 / det;
  Jinv[0] = (Jm(1, 1) * Jm(2, 2) - Jm(1, 2) * Jm(2, 1)) * id;
  Jinv[1] = (Jm(0, 2) * Jm(2, 1) - Jm(0, 1) * Jm(2, 2)) * id;
  Jinv[2] = (Jm(0, 1) * Jm(1, 2) - Jm(0, 2) * Jm(1, 1)) * id;
  Jinv[3] = (Jm(1, 2) * Jm(2, 0) - Jm(1, 0) * Jm(2, 2)) * id;
  Jinv[4] = (Jm(0, 0) * Jm(2, 2) - Jm(0, 2) * Jm(2, 0)) * id;
  Jinv[5] = (Jm(0, 2) * Jm(1, 0) - Jm(0, 0) * Jm(1, 2)) * id;
  Jinv[6] = (Jm(1, 0) * Jm(2, 1) - Jm(1, 1) * Jm(2, 0)) * id;
  Jinv[7] = (Jm(0, 1) * Jm(2, 0) - Jm(0, 0) * Jm(2, 1)) * id;
  Jinv[8] = (Jm(0, 0) * Jm(1, 1) - Jm(0, 1) * Jm(1, 0)) * id;
}

// Jacobian modificators (src/domain/Axisymmetry.cpp:33-56,
// AxisymmetryShell.cpp:37-95, PolarShell.cpp:37-93, CylindricalShell.cpp:37-101,
// SphericalShell.cpp:37-95): at the physical point x the Jacobian
// (J[3c + r] = dx_r/du_c) becomes J * jac with jac[m][l] = dx'_l/dx_m of the
// shell map x -> x', and det is multiplied by det(jac). The shells stretch
// the radius r in [rmin, rmax) with f = (rmin (rmax - rmin) / (r (rmax - r)))^k
// and theta = k (rmax - 2r) / (rmax - r): jac = f (I - theta dr dr^T) in the
// stretched directions. Returns false for a radius outside [rmin, rmax] (10
// machine epsilons of slack); a radius at rmax is pulled inside by 10 epsilons.
__host__ __device__ inline bool applyJacMod(const DevJacMod &m, const double *x, double *J, double &det) {
  constexpr double eps = 2.220446049250313e-16;  // double machine epsilon
  if (m.kind == FG_JACMOD_AXISYMMETRY) {
    const double r = x[0] == 0.0 ? eps : x[0];
    J[8] = r;
    det *= r;
    return true;
  }
  double d[3] = {0.0, 0.0, 0.0};
  int nd = 3;
  if (m.kind == FG_JACMOD_AXISYMMETRY_SHELL) {
    d[0] = x[0];
    d[1] = x[1] - m.center[1];
    nd = 2;
  } else if (m.kind == FG_JACMOD_POLAR_SHELL) {
    d[0] = x[0] - m.center[0];
    d[1] = x[1] - m.center[1];
    nd = 2;
  } else {
    for (int j = 0; j < 3; ++j) d[j] = (m.kind == FG_JACMOD_CYLINDRICAL_SHELL && j == m.axis) ? 0.0 : x[j] - m.center[j];
  }
  double R = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  if (R < m.rmin - 10.0 * eps || R > m.rmax + 10.0 * eps) return false;
  if (R >= m.rmax) R = m.rmax - 10.0 * eps;
  double g[3];
  for (int j = 0; j < 3; ++j) g[j] = d[j] / R;
  const double base = (m.rmin * (m.rmax - m.rmin)) / (R * (m.rmax - R));
  double f = 1.0;
  for (int k = 0; k < m.exponent; ++k) f *= base;
  const double theta = m.exponent * (m.rmax - 2.0 * R) / (m.rmax - R);
  double jac[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) jac[a][b] = f * ((a == b ? 1.0 : 0.0) - theta * g[a] * g[b]);
  double J2[9];
  if (nd == 3) {
    if (m.kind == FG_JACMOD_CYLINDRICAL_SHELL) jac[m.axis][m.axis] = 1.0;
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) J2[3 * k + l] = J[3 * k] * jac[0][l] + J[3 * k + 1] * jac[1][l] + J[3 * k + 2] * jac[2][l];
    det *= m.kind == FG_JACMOD_CYLINDRICAL_SHELL ? f * f * (1.0 - theta) : f * f * f * (1.0 - theta);
  } else {
    for (int k = 0; k < 2; ++k)
      for (int l = 0; l < 2; ++l) J2[3 * k + l] = J[3 * k] * jac[0][l] + J[3 * k + 1] * jac[1][l];
    J2[2] = J2[5] = J2[6] = J2[7] = 0.0;
    if (m.kind == FG_JACMOD_POLAR_SHELL) {
      J2[8] = 1.0;
      det *= f * f * (1.0 - theta);
    } else {
      const double S = x[0] == 0.0 ? eps : x[0];
      J2[8] = S * f;
      det *= S * (f * f * f * (1.0 - theta));
    }
  }
  for (int k = 0; k < 9; ++k) J[k] = J2[k];
  return true;
}

// Lane-0 geometry of integration point q for the terms of modificator group
// g: J0/det0 hold the unmodified Jacobian (formed once for affine elements),
// J/det/Jinv the one the group's terms use, xq the physical point.
__device__ inline void pointGeometry(const PlanDev &p, const DevTerms *terms, int g, int q, const double *X, double *J0, double &det0,
                                     double *J, double &det, double *Jinv, double *xq) {
  if (q == 0 || !p.affine) det0 = jacobian(p.dim, p.nn, X, p.geoGrad + (size_t)q * p.nn * 3, J0);
  xq[0] = xq[1] = xq[2] = 0.0;
  for (int k = 0; k < p.nn; ++k) {
    const double v = p.geoVal[q * p.nn + k];
    xq[0] += v * X[3 * k];
    xq[1] += v * X[3 * k + 1];
    xq[2] += v * X[3 * k + 2];
  }
  const DevJacMod &m = terms->mods[g];
  if (m.kind != FG_JACMOD_NONE || q == 0 || !p.affine || terms->nMod > 1) {
    for (int k = 0; k < 9; ++k) J[k] = J0[k];
    det = det0;
    if (m.kind != FG_JACMOD_NONE && !applyJacMod(m, xq, J, det)) atomicOr(p.jmErr, 1);
    jacobianInverse(J, det, Jinv);
  }
}


}  // namespace femg
