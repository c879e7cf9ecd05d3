// common.cuh -- shared helpers for the HDoG sm_103a kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/hdog.h"

namespace hdog {

// Volume geometry of one substack: x fastest, then y, then z (linear index
// (z*H + y)*W + x, the layout of the reference's device buffers).
struct Geom {
  int W, H, D;
  __host__ __device__ int64_t n() const { return (int64_t)W * H * D; }
  __host__ __device__ int64_t plane() const { return (int64_t)W * H; }
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Packed u16 pair of a running min / max: low half = min (erosion), high half =
// 65535 - max (dilation), so a single __vminu2 combines both halves.
__device__ __forceinline__ uint32_t pack_mm(uint32_t lo, uint32_t hi) { return lo | ((hi ^ 0xFFFFu) << 16); }
__device__ __forceinline__ uint32_t mm_combine(uint32_t a, uint32_t b) { return __vminu2(a, b); }
__device__ __forceinline__ uint32_t mm_lo(uint32_t v) { return v & 0xFFFFu; }
__device__ __forceinline__ uint32_t mm_hi(uint32_t v) { return (v >> 16) ^ 0xFFFFu; }

// Two IEEE round-to-nearest float adds / FMAs in one instruction (sm_100+ f32x2).  Each
// lane rounds exactly like a scalar FADD / FFMA, so results equal the scalar chain.
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  unsigned long long ra = *reinterpret_cast<unsigned long long *>(&a);
  unsigned long long rb = *reinterpret_cast<unsigned long long *>(&b);
  unsigned long long rd;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
  return *reinterpret_cast<float2 *>(&rd);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  unsigned long long ra = *reinterpret_cast<unsigned long long *>(&a);
  unsigned long long rb = *reinterpret_cast<unsigned long long *>(&b);
  unsigned long long rc = *reinterpret_cast<unsigned long long *>(&c);
  unsigned long long rd;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(ra), "l"(rb), "l"(rc));
  return *reinterpret_cast<float2 *>(&rd);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  unsigned long long ra = *reinterpret_cast<unsigned long long *>(&a);
  unsigned long long rb = *reinterpret_cast<unsigned long long *>(&b);
  unsigned long long rd;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
  return *reinterpret_cast<float2 *>(&rd);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  unsigned long long ra = *reinterpret_cast<unsigned long long *>(&a);
  unsigned long long rb = *reinterpret_cast<unsigned long long *>(&b);
  unsigned long long rd;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
  return *reinterpret_cast<float2 *>(&rd);
}

// Float max in a monotone unsigned encoding, for atomicMax on region maxima.
__device__ __forceinline__ uint32_t f2ord(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float ord2f(uint32_t o) {
  uint32_t u = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

// One central difference as gradientRowsKernel (:22-74) writes it:
// sum = 0; sum += s[+1]; sum -= s[-1]; sum *= 0.5f.
__device__ __forceinline__ float cdiff(float plus, float minus) {
  return __fmul_rn(__fsub_rn(__fadd_rn(0.0f, plus), minus), 0.5f);
}

// Sylvester test of PositiveDefiniteKernel (Hessian3DFilter_element.cu:295-323) with
// every rounding written out, in the form nvcc gives the reference's expression
// (pinned against the reference binary on crafted near-singular matrices):
//   xx < 0
//   xx*yy > xy*xy              (`a - b > 0` folded to `a > b`, both products rounded)
//   t = fma(xx*yy, zz, (2xy*yz)*xz); t = fma(-(xx*yz), yz, t); t = fma(-(yy*xz), xz, t)
//   t < (zz*xy)*xy             (the last subtraction of the determinant folded into `< 0`)
// All three conditions are evaluated and combined without short-circuit: the products
// have no side effects, so the result is the same, and the tile kernels test four voxels
// per thread without a divergent branch per voxel.
__device__ __forceinline__ bool pd_test(float xx, float xy, float xz, float yy, float yz, float zz) {
  const float p = __fmul_rn(xx, yy);
  const float q = __fmul_rn(__fmul_rn(2.0f, xy), yz);
  float t = __fmaf_rn(p, zz, __fmul_rn(q, xz));
  t = __fmaf_rn(-__fmul_rn(xx, yz), yz, t);
  t = __fmaf_rn(-__fmul_rn(yy, xz), xz, t);
  return (xx < 0.0f) & (p > __fmul_rn(xy, xy)) & (t < __fmul_rn(__fmul_rn(zz, xy), xy));
}

// The six Hessian elements at voxel (x, y, z) straight from global memory, with the
// same zero-halo rule as the tiled kernel: f outside the volume is 0 and a first
// derivative at a position outside the volume is 0.  Order xx, xy, xz, yy, yz, zz.
__device__ __forceinline__ float dog_ld(const float *f, int W, int H, int D, int x, int y, int z) {
  return (x >= 0 && y >= 0 && z >= 0 && x < W && y < H && z < D) ? __ldg(f + ((int64_t)z * H + y) * W + x) : 0.0f;
}
__device__ __forceinline__ float grad1(const float *f, int W, int H, int D, int x, int y, int z, int dx,
                                       int dy, int dz) {
  if (x < 0 || y < 0 || z < 0 || x >= W || y >= H || z >= D) return 0.0f;
  return cdiff(dog_ld(f, W, H, D, x + dx, y + dy, z + dz), dog_ld(f, W, H, D, x - dx, y - dy, z - dz));
}
__device__ __forceinline__ void hessian_at(const float *f, int W, int H, int D, int x, int y, int z,
                                           float h[6]) {
  h[0] = cdiff(grad1(f, W, H, D, x + 1, y, z, 1, 0, 0), grad1(f, W, H, D, x - 1, y, z, 1, 0, 0));
  h[1] = cdiff(grad1(f, W, H, D, x, y + 1, z, 1, 0, 0), grad1(f, W, H, D, x, y - 1, z, 1, 0, 0));
  h[2] = cdiff(grad1(f, W, H, D, x, y, z + 1, 1, 0, 0), grad1(f, W, H, D, x, y, z - 1, 1, 0, 0));
  h[3] = cdiff(grad1(f, W, H, D, x, y + 1, z, 0, 1, 0), grad1(f, W, H, D, x, y - 1, z, 0, 1, 0));
  h[4] = cdiff(grad1(f, W, H, D, x, y, z + 1, 0, 1, 0), grad1(f, W, H, D, x, y, z - 1, 0, 1, 0));
  h[5] = cdiff(grad1(f, W, H, D, x, y, z + 1, 0, 0, 1), grad1(f, W, H, D, x, y, z - 1, 0, 0, 1));
}

// Region float sums accumulate as 64-bit fixed point with 36 fractional bits: integer
// atomics are associative, so the sums (and every record) are identical run to run.
constexpr double kFixScale = 68719476736.0;          // 2^36
constexpr double kFixInv = 1.0 / 68719476736.0;
// v * 2^36 is exact in float (a power-of-two scaling), so rounding it to an integer
// gives the same fixed-point value as the double product, without the FP64 pipe.
__device__ __forceinline__ unsigned long long to_fix(float v) {
  return (unsigned long long)__float2ll_rn(v * 68719476736.0f);
}
__host__ __device__ __forceinline__ double from_fix(unsigned long long v) { return (double)(long long)v * kFixInv; }

constexpr int kMaxTaps = 80;   // MAX_KERNEL_LENGTH of the reference DoG taps

// Gaussian taps of both DoG scales in constant memory: [0] small xy, [1] small z,
// [2] large xy, [3] large z (the c_Kernel layout of the reference).
struct DogTaps {
  float k[4][kMaxTaps];
  int r[4];
  float normalizer;
};

// ---- mbarrier / TMA helpers (sm_90+ PTX).  Every wait is bounded: after kWaitLimit
// polls it gives up and the caller records HDOG_ERR_TIMEOUT.
constexpr long long kWaitLimit = 1ll << 26;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done = 0;
  for (long long it = 0; it < kWaitLimit && !done; it++) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
  }
  return done != 0;
}

// One arrival on bar (release: the caller's shared-memory reads before it are ordered
// before whatever a waiter does after the phase completes).
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
      : "memory");
}

// One box of a 4-D tensor map (x, y, z, substack) into shared memory, completing on bar.
__device__ __forceinline__ void tma_load_4d(const void *map, void *dst, uint64_t *bar, int x, int y, int z, int s,
                                            uint32_t bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(s), "r"(smem_u32(bar))
      : "memory");
}

// Optional per-kernel timing: when a context enables it, each kernel launch is
// bracketed by CUDA events recorded on the launching stream.
struct KernelTimer {
  virtual void begin(const char *name, cudaStream_t s) = 0;
  virtual void end(cudaStream_t s) = 0;
  virtual ~KernelTimer() {}
};
extern thread_local KernelTimer *g_timer;

}  // namespace hdog

#define KT_BEGIN(name, s)                            \
  do {                                               \
    if (::hdog::g_timer) ::hdog::g_timer->begin(name, s); \
  } while (0)
#define KT_END(s)                                    \
  do {                                               \
    if (::hdog::g_timer) ::hdog::g_timer->end(s);    \
  } while (0)
// Launch `kernel<<<args>>>(...)` between timing events named after the kernel.
#define KLAUNCH(name, s, launch) \
  do {                           \
    KT_BEGIN(name, s);           \
    launch;                      \
    KT_END(s);                   \
  } while (0)

#define HDOG_CUDA_TRY(expr)                                 \
  do {                                                      \
    cudaError_t e__ = (expr);                               \
    if (e__ != cudaSuccess) return hdog_set_cuda_error(e__, #expr); \
  } while (0)

extern "C" int hdog_set_cuda_error(cudaError_t e, const char *what);
