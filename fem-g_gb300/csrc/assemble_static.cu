// fg_assemble_fp64_static: the FP64 assembly of fg_assemble_fp64 with its
// element-matrix and element-vector scratch in a fixed, file-scope device
// array instead of plan-owned buffers grown with cudaMalloc, for callers that
// may not allocate device memory once their set-up is done.
//
// The call allocates nothing: terms come from fg_plan_bind_terms, outputs and
// Dirichlet values must already be device memory, and the element kernels and
// the row-owner gather run on the scratch array. Its address is resolved once
// per device (cudaGetSymbolAddress, with that device current) in the first
// call made on the device; make that first call before any stream capture.
// The array is shared by every plan on a device, so two calls in flight at
// the same time on one device (other streams, other host threads) race on it.
#include <mutex>

#include "common.cuh"

namespace femg {

constexpr size_t kStaticScratchBytes = FG_STATIC_SCRATCH_BYTES;  // 64 MiB per device
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_staticScratch[kStaticScratchBytes];

static std::mutex g_staticMutex;
static void *g_staticPtr[kStaticMaxDevices];

// Address of the scratch array on the current device, resolved on first use.
static int staticScratch(void **out) {
  int dev = 0;
  FG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kStaticMaxDevices) {
    setLastError("fg_assemble_fp64_static: device ordinal beyond the static table");
    return FG_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_staticMutex);
  if (!g_staticPtr[dev]) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_staticScratch);
    if (e != cudaSuccess || !ptr) {
      cudaGetLastError();
      setLastError(std::string("fg_assemble_fp64_static: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      return FG_ERR_CUDA;
    }
    g_staticPtr[dev] = ptr;
  }
  *out = g_staticPtr[dev];
  return FG_OK;
}

}  // namespace femg

using namespace femg;

extern "C" int fg_assemble_fp64_static(fg_plan *plan, const double *dirichlet, double *csr_values, double *rhs, void *stream) {
  if (!plan) return FG_ERR_ARG;
  if (!plan->hasBound) {
    setLastError("fg_assemble_fp64_static: terms must be bound with fg_plan_bind_terms first");
    return FG_ERR_ARG;
  }
  if (!csr_values || !isDevicePointer(csr_values) || (rhs && !isDevicePointer(rhs))) {
    setLastError("fg_assemble_fp64_static: csr_values and rhs must be device memory");
    return FG_ERR_ARG;
  }
  const PlanDev &p = plan->d;
  if (int st0 = coupledLiftCheck(plan, rhs)) return st0;
  const double *uD = nullptr;
  if (p.nFixed > 0) {
    if (!dirichlet || !isDevicePointer(dirichlet)) {
      setLastError("fg_assemble_fp64_static: the system has fixed DOFs: dirichlet must be device memory");
      return FG_ERR_ARG;
    }
    uD = dirichlet;
  }
  const DevTerms &dt = plan->bound;
  const int ncomp = dt.complexKe ? 2 : 1;
  // [E][ncomp][n][nc] element matrices, then [E][n] complex element vectors at
  // the next 256-byte boundary. Every entry is written by the element kernels
  // before the gather reads it, so no part of the array is cleared.
  const size_t keBytes = (size_t)p.E * ncomp * p.n * p.nc * sizeof(double);
  const bool withBe = dt.hasSource && rhs;
  const size_t beOff = (keBytes + 255) / 256 * 256;
  const size_t need = withBe ? beOff + (size_t)p.E * p.n * 16 : keBytes;
  if (need > kStaticScratchBytes) {
    setLastError("fg_assemble_fp64_static: element scratch of " + std::to_string(need) + " bytes exceeds the " +
                 std::to_string(kStaticScratchBytes) + "-byte static array");
    return FG_ERR_UNSUPPORTED;
  }
  void *base = nullptr;
  int st = staticScratch(&base);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  double *ke = (double *)base;
  double *be = withBe ? (double *)((unsigned char *)base + beOff) : nullptr;
  if (p.E > 0) {
    if ((st = launchElementFp64(plan, dt, plan->boundDev, ke, be, s))) return st;
  }
  return launchGather(plan, ke, dt.complexKe, 0, keRect(p.n, p.nc), be, uD, csr_values, rhs, s);
}
