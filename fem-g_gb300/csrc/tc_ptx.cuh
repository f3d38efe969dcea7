// Device helpers of the tensor-core kernels: the TF32 split of FP64 values
// and inline PTX for tcgen05 (TMEM allocation, MMA, commit, loads), mbarriers
// and TMA / bulk copies. Included inside namespace femg.
#pragma once

constexpr long long kWaitCycles = 4000000000LL;  // ~2 s bound on any device-side wait

// ------------------------------------------------------------ TF32 split

// round-to-nearest (ties away from zero) of an fp32 value to TF32 (10 mantissa bits)
__host__ __device__ inline float tf32Round(float x) {
  uint32_t b;
  memcpy(&b, &x, 4);
  if ((b & 0x7F800000u) == 0x7F800000u) return x;  // inf / nan
  b = (b + 0x1000u) & 0xFFFFE000u;
  float r;
  memcpy(&r, &b, 4);
  return r;
}

__host__ __device__ inline void splitTf32(double x, float &hi, float &lo) {
  hi = tf32Round((float)x);
  lo = tf32Round((float)(x - (double)hi));
}

// The same split on the device with one FP64 operation (GB300's FP64 pipe is
// narrow): x rounded to 11 significant bits on its bit pattern (ties away
// from zero, the carry runs into the exponent), the exact remainder rounded
// the same way, each narrowed to float by moving the exponent.
__device__ inline double roundTf32Bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return __longlong_as_double((long long)((b + (1ull << 41)) & ~((1ull << 42) - 1ull)));
}
__device__ inline float narrowTf32(double h) {  // h has at most 11 significant bits
  const unsigned long long b = (unsigned long long)__double_as_longlong(h);
  const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
  if (e <= 0 || e >= 255) return (float)h;  // zero, float subnormal, overflow, inf/nan
  return __uint_as_float(((uint32_t)(b >> 32) & 0x80000000u) | ((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7FFFFFu));
}
__device__ inline void splitTf32Dev(double x, float &hi, float &lo) {
  const double h = roundTf32Bits(x);
  hi = narrowTf32(h);
  lo = narrowTf32(roundTf32Bits(x - h));  // x - h is exact
}

// ------------------------------------------------------- PTX primitives

__device__ inline uint32_t smemAddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, no swizzle, 8x16B core matrices
__device__ inline uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;               // base offset 0, relative LBO, SWIZZLE_NONE
}

// instruction descriptor: kind::tf32, D fp32, A/B tf32 K-major, M x N
__device__ inline uint32_t idescTf32(int M, int N) {
  uint32_t d = 0;
  d |= 1u << 4;                       // D format F32
  d |= 2u << 7;                       // A format TF32
  d |= 2u << 10;                      // B format TF32
  d |= (uint32_t)(N >> 3) << 17;
  d |= (uint32_t)(M >> 4) << 24;
  return d;
}

__device__ inline void tmemAlloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(dst)), "r"(ncols) : "memory");
}
__device__ inline void tmemRelinquish() { asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory"); }
__device__ inline void tmemDealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ inline void mmaTf32(uint32_t dTmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dTmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ inline void mmaCommit(uint64_t *mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(mbar)) : "memory");
}
__device__ inline void tcFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ inline void tcFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ inline void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ inline void mbarInit(uint64_t *mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(mbar)), "r"(count) : "memory");
}
__device__ inline void fenceMbarInit() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ inline bool mbarTryWait(uint64_t *mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smemAddr(mbar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; false on timeout
__device__ inline bool mbarWait(uint64_t *mbar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbarTryWait(mbar, parity))
    if (clock64() - t0 > kWaitCycles) return false;
  return true;
}
// the same with a caller-given bound in SM cycles; 0 gives up at once
__device__ inline bool mbarWaitFor(uint64_t *mbar, uint32_t parity, long long cycles) {
  if (cycles <= 0) return false;
  const long long t0 = clock64();
  while (!mbarTryWait(mbar, parity))
    if (clock64() - t0 > cycles) return false;
  return true;
}
// TMA: the arrival that announces `bytes` of transaction on the barrier,
// and a 2D tiled load of box {4 floats, 128 rows} at (x, y) completing on it
__device__ inline void mbarExpectTx(uint64_t *mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(mbar)), "r"(bytes) : "memory");
}
__device__ inline void tmaLoad2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint64_t *mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smemAddr(mbar))
      : "memory");
}

// TMA bulk copy (no tensor map) of `bytes` (a multiple of 16, both
// addresses 16-byte aligned) completing on the barrier
__device__ inline void bulkLoad(uint32_t dst, const void *src, uint32_t bytes, uint64_t *mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smemAddr(mbar))
               : "memory");
}

__device__ inline void tmemLoad16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ inline void tmemLoad32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

// cp.async of 16 bytes (srcBytes < 16: the rest zero-filled), commit and wait
__device__ inline void cpAsync16(uint32_t dst, const void *src, uint32_t srcBytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(srcBytes) : "memory");
}
__device__ inline void cpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ inline void cpAsyncWaitAll() { asm volatile("cp.async.wait_all;" ::: "memory"); }
