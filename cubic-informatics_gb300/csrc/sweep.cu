// sweep.cu -- fused DoG + Hessian + negative-definite test, one z-sweep per xy tile, sm_103a.
//
// Reference: src/3D/DoG3DFilter.cu (DoG3DFilter :431-437: x -> y -> z separable Gaussians
// with zero borders, `(small - large) * normalizer`) and src/3D/Hessian3DFilter_element.cu
// (HessianPositiveDefiniteWithElement :355-388: gradients of gradients with zero halos,
// Sylvester test).  The reference runs 16 full-volume passes here and keeps the DoG and
// six Hessian planes in memory; this kernel reads the normalized volume once and writes
// the uint8 mask plus a compact list of the foreground voxels' Hessian elements.
//
// The generic kernel (k_dog_hess, any tap radii) gives a block a 64 x 16 output tile and
// sweeps z over the whole substack:
//   * each normalized slice (tile + halo, zero outside the volume) arrives by TMA
//     (cp.async.bulk.tensor, mbarrier-completed, double buffered) while the previous one
//     is filtered;
//   * x and y passes run in shared memory over the tile extended by the Hessian's
//     2-voxel halo; both scales travel in one f32x2 (small .x, large .y);
//   * the z pass is a per-thread shift register of 2*RZ+1 partial sums: each new y-pass
//     value is added to every pending output in ascending tap order, so every DoG value
//     is the reference's FMA chain;
//   * finished DoG slices go to a 5-slice ring, from which the Hessian of slice z-2 is
//     formed with the reference's zero-halo gradients and tested.
// Every wait on the TMA barrier is bounded; a timeout sets HDOG_ERR_TIMEOUT and the
// kernel finishes without further waits.
#include <cuda.h>

#include <algorithm>

#include <type_traits>

#include "kernels.cuh"

namespace hdog {

constexpr int kSX = 64, kSY = 16;                 // mask tile
constexpr int kEX = kSX + 4, kEY = kSY + 4;       // DoG tile with the Hessian halo
constexpr int kSweepThreads = 704;                // 22 warps
constexpr int kXQuads = kEX / 4;                  // 17 four-wide x-pass items per row

__host__ __device__ inline int sweep_hx(int rxy) { return ((rxy + 2 + 3) / 4) * 4; }   // aligned x halo
__host__ __device__ inline int sweep_bw(int rxy) { return kSX + 2 * sweep_hx(rxy); }
__host__ __device__ inline int sweep_bh(int rxy) { return kSY + 4 + 2 * rxy; }

size_t sweep_smem_bytes(int rxy) {
  const size_t in = ((size_t)sweep_bw(rxy) * sweep_bh(rxy) * 4 + 127) / 128 * 128;
  const size_t xb = (size_t)sweep_bh(rxy) * kEX * sizeof(float2);
  const size_t ring = (size_t)5 * kEY * kEX * sizeof(float);
  return 2 * in + xb + ring + 64;
}

// One normalized slice (box bw x bh at (x, y, z, s)) into shared memory.
__device__ __forceinline__ void tma_slice(const CUtensorMap *map, float *dst, uint64_t *bar, int x, int y, int z, int s,
                                          uint32_t bytes) {
  tma_load_4d(map, dst, bar, x, y, z, s, bytes);
}

template <int RZ>
__global__ void __launch_bounds__(kSweepThreads, 1)
    k_dog_hess(const __grid_constant__ CUtensorMap map, const __grid_constant__ DogTaps T, const Sub *subs,
               const float *norm, uint8_t *mask, FgEntry *fg, int32_t *fg_idx, unsigned long long *fg_count,
               int *status) {
  constexpr int WIN = 2 * RZ + 1;
  extern __shared__ __align__(128) unsigned char smem[];
  const Sub S = subs[blockIdx.y];
  const int ntx = (S.W + kSX - 1) / kSX, nty = (S.H + kSY - 1) / kSY;
  if ((int64_t)blockIdx.x >= (int64_t)ntx * nty) return;
  const int x0 = (int)(blockIdx.x % ntx) * kSX, y0 = (int)(blockIdx.x / ntx) * kSY;
  const int ra = T.r[0], rb = T.r[2], rxy = max(ra, rb);
  const int za = T.r[1], zb = T.r[3];
  const int hx = sweep_hx(rxy), bw = sweep_bw(rxy), bh = sweep_bh(rxy);
  const size_t in_bytes = ((size_t)bw * bh * 4 + 127) / 128 * 128;
  float *inb[2] = {reinterpret_cast<float *>(smem), reinterpret_cast<float *>(smem + in_bytes)};
  float2 *xb = reinterpret_cast<float2 *>(smem + 2 * in_bytes);
  float *ring = reinterpret_cast<float *>(smem + 2 * in_bytes + (size_t)bh * kEX * sizeof(float2));
  uint64_t *bar = reinterpret_cast<uint64_t *>(ring + 5 * kEY * kEX);
  const int t = threadIdx.x;
  const int D = S.D, W = S.W, H = S.H;
  const int64_t WH = (int64_t)W * H;
  if (t == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const uint32_t tma_bytes = (uint32_t)(bw * bh * 4);
  const int tx = x0 - hx, ty = y0 - 2 - rxy;
  bool ok = true;

  // y / z pass ownership: columns (cx, cy) and (cx, cy + 1) of the extended tile
  const bool yz_thread = t < kEX * (kEY / 2);
  const int cx = t % kEX, cy = 2 * (t / kEX);
  const int gx = x0 - 2 + cx, gy0 = y0 - 2 + cy;
  float2 acc0[WIN], acc1[WIN];
#pragma unroll
  for (int s = 0; s < WIN; s++) { acc0[s] = make_float2(0.f, 0.f); acc1[s] = make_float2(0.f, 0.f); }

  for (int zi = -RZ; zi <= D + 1 + RZ; zi++) {
    const bool have = zi >= 0 && zi < D;
    if (have && ok) {
      if (!mbar_wait(&bar[zi & 1], (zi >> 1) & 1)) {
        ok = false;
        atomicExch(status, HDOG_ERR_TIMEOUT);
      }
    }
    if (t == 0 && ok && zi + 1 >= 0 && zi + 1 < D)
      tma_slice(&map, inb[(zi + 1) & 1], &bar[(zi + 1) & 1], tx, ty, zi + 1, blockIdx.y, tma_bytes);
    // ---- x pass: four outputs per item, sliding window over the smem row
    if (have && t < bh * kXQuads) {
      const int row = t / kXQuads, q = t % kXQuads;
      const float *in = inb[zi & 1] + row * bw + (4 * q - 2 + hx);   // input of output ex = 4q at offset 0
      float2 a[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
      float w0 = in[-rxy], w1 = in[-rxy + 1], w2 = in[-rxy + 2];
      for (int j = -rxy; j <= rxy; j++) {
        const float w3 = in[j + 3];
        const bool aa = j >= -ra && j <= ra, ab = j >= -rb && j <= rb;
        if (aa && ab) {
          const float2 kk = make_float2(T.k[0][ra - j], T.k[2][rb - j]);
          a[0] = fma2(kk, make_float2(w0, w0), a[0]);
          a[1] = fma2(kk, make_float2(w1, w1), a[1]);
          a[2] = fma2(kk, make_float2(w2, w2), a[2]);
          a[3] = fma2(kk, make_float2(w3, w3), a[3]);
        } else if (ab) {
          const float kk = T.k[2][rb - j];
          a[0].y = __fmaf_rn(kk, w0, a[0].y);
          a[1].y = __fmaf_rn(kk, w1, a[1].y);
          a[2].y = __fmaf_rn(kk, w2, a[2].y);
          a[3].y = __fmaf_rn(kk, w3, a[3].y);
        } else if (aa) {
          const float kk = T.k[0][ra - j];
          a[0].x = __fmaf_rn(kk, w0, a[0].x);
          a[1].x = __fmaf_rn(kk, w1, a[1].x);
          a[2].x = __fmaf_rn(kk, w2, a[2].x);
          a[3].x = __fmaf_rn(kk, w3, a[3].x);
        }
        w0 = w1; w1 = w2; w2 = w3;
      }
      float2 *o = xb + row * kEX + 4 * q;
      o[0] = a[0]; o[1] = a[1]; o[2] = a[2]; o[3] = a[3];
    }
    __syncthreads();
    // ---- y pass (two outputs), z pass (shift register), emit DoG slice zi - RZ
    if (yz_thread) {
      float2 g0 = make_float2(0.f, 0.f), g1 = make_float2(0.f, 0.f);
      if (have) {
        const float2 *col = xb + (cy + rxy) * kEX + cx;
        float2 v0 = col[-rxy * kEX];
        for (int j = -rxy; j <= rxy; j++) {
          const float2 v1 = col[(j + 1) * kEX];
          const bool aa = j >= -ra && j <= ra, ab = j >= -rb && j <= rb;
          if (aa && ab) {
            const float2 kk = make_float2(T.k[0][ra - j], T.k[2][rb - j]);
            g0 = fma2(kk, v0, g0);
            g1 = fma2(kk, v1, g1);
          } else if (ab) {
            const float kk = T.k[2][rb - j];
            g0.y = __fmaf_rn(kk, v0.y, g0.y);
            g1.y = __fmaf_rn(kk, v1.y, g1.y);
          } else if (aa) {
            const float kk = T.k[0][ra - j];
            g0.x = __fmaf_rn(kk, v0.x, g0.x);
            g1.x = __fmaf_rn(kk, v1.x, g1.x);
          }
          v0 = v1;
        }
      }
      // slot s holds output zo = zi - RZ + s; this input is tap d = RZ - s of it
#pragma unroll
      for (int s = 0; s < WIN; s++) {
        const int d = RZ - s;
        const bool aa = d >= -za && d <= za, ab = d >= -zb && d <= zb;
        if (aa && ab) {
          const float2 kk = make_float2(T.k[1][za - d], T.k[3][zb - d]);
          acc0[s] = fma2(kk, g0, acc0[s]);
          acc1[s] = fma2(kk, g1, acc1[s]);
        } else if (ab) {
          const float kk = T.k[3][zb - d];
          acc0[s].y = __fmaf_rn(kk, g0.y, acc0[s].y);
          acc1[s].y = __fmaf_rn(kk, g1.y, acc1[s].y);
        } else if (aa) {
          const float kk = T.k[1][za - d];
          acc0[s].x = __fmaf_rn(kk, g0.x, acc0[s].x);
          acc1[s].x = __fmaf_rn(kk, g1.x, acc1[s].x);
        }
      }
      const int zo = zi - RZ;
      if (zo >= -2 && zo <= D + 1) {
        const bool zin = zo >= 0 && zo < D;
        const bool in0 = zin && gx >= 0 && gx < W && gy0 >= 0 && gy0 < H;
        const bool in1 = zin && gx >= 0 && gx < W && gy0 + 1 >= 0 && gy0 + 1 < H;
        float *r = ring + ((zo + 5) % 5) * kEY * kEX + cy * kEX + cx;
        r[0] = in0 ? __fmul_rn(__fsub_rn(acc0[0].x, acc0[0].y), T.normalizer) : 0.0f;
        r[kEX] = in1 ? __fmul_rn(__fsub_rn(acc1[0].x, acc1[0].y), T.normalizer) : 0.0f;
      }
#pragma unroll
      for (int s = 0; s < WIN - 1; s++) { acc0[s] = acc0[s + 1]; acc1[s] = acc1[s + 1]; }
      acc0[WIN - 1] = make_float2(0.f, 0.f);
      acc1[WIN - 1] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    // ---- Hessian + PD of slice zh = zi - RZ - 2 (DoG slices zh-2 .. zh+2 are in the ring)
    const int zh = zi - RZ - 2;
    if (zh >= 0 && zh < D) {
      int nfg = 0;
      int64_t idx[2] = {0, 0};
      float hv[2][6];
      bool fgv[2] = {false, false};
      if (t < kSX * (kSY / 2)) {
        const int hx0 = t % kSX, hy0 = 2 * (t / kSX);
        // tiles whose every voxel has all in-plane neighbours inside the volume take the
        // fast path: only the z neighbours can fall outside
        const bool interior = x0 >= 1 && x0 + kSX < W && y0 >= 1 && y0 + kSY < H;
        if (interior) {
          const float *P0 = ring + (zh % 5) * kEY * kEX;
          const float *P1 = ring + ((zh + 1) % 5) * kEY * kEX;
          const float *P2 = ring + ((zh + 2) % 5) * kEY * kEX;
          const float *M1 = ring + ((zh + 4) % 5) * kEY * kEX;
          const float *M2 = ring + ((zh + 3) % 5) * kEY * kEX;
          const bool zup = zh + 1 < D, zdn = zh >= 1;
          for (int u = 0; u < 2; u++) {
            const int c = (hy0 + u + 2) * kEX + (hx0 + 2);
            float *h = hv[u];
            h[0] = cdiff(cdiff(P0[c + 2], P0[c]), cdiff(P0[c], P0[c - 2]));
            h[1] = cdiff(cdiff(P0[c + kEX + 1], P0[c + kEX - 1]), cdiff(P0[c - kEX + 1], P0[c - kEX - 1]));
            h[2] = cdiff(zup ? cdiff(P1[c + 1], P1[c - 1]) : 0.0f, zdn ? cdiff(M1[c + 1], M1[c - 1]) : 0.0f);
            h[3] = cdiff(cdiff(P0[c + 2 * kEX], P0[c]), cdiff(P0[c], P0[c - 2 * kEX]));
            h[4] = cdiff(zup ? cdiff(P1[c + kEX], P1[c - kEX]) : 0.0f, zdn ? cdiff(M1[c + kEX], M1[c - kEX]) : 0.0f);
            h[5] = cdiff(zup ? cdiff(P2[c], P0[c]) : 0.0f, zdn ? cdiff(P0[c], M2[c]) : 0.0f);
            const bool pd = pd_test(h[0], h[1], h[2], h[3], h[4], h[5]);
            idx[u] = zh * WH + (int64_t)(y0 + hy0 + u) * W + (x0 + hx0);
            mask[S.vox + idx[u]] = pd ? 1 : 0;
            fgv[u] = pd && idx[u] != 0;
            nfg += fgv[u];
          }
        } else {
          for (int u = 0; u < 2; u++) {
            const int lx = hx0, ly = hy0 + u;
            const int X = x0 + lx, Y = y0 + ly;
            if (X >= W || Y >= H) continue;
            const int ex = lx + 2, ey = ly + 2;
            auto Dv = [&](int ddx, int ddy, int ddz) -> float {
              return ring[((zh + ddz + 5) % 5) * kEY * kEX + (ey + ddy) * kEX + (ex + ddx)];
            };
            auto in_vol = [&](int ddx, int ddy, int ddz) -> bool {
              const int xx = X + ddx, yy = Y + ddy, zz = zh + ddz;
              return xx >= 0 && xx < W && yy >= 0 && yy < H && zz >= 0 && zz < D;
            };
            auto GX = [&](int ddx, int ddy, int ddz) -> float {
              return in_vol(ddx, ddy, ddz) ? cdiff(Dv(ddx + 1, ddy, ddz), Dv(ddx - 1, ddy, ddz)) : 0.0f;
            };
            auto GY = [&](int ddx, int ddy, int ddz) -> float {
              return in_vol(ddx, ddy, ddz) ? cdiff(Dv(ddx, ddy + 1, ddz), Dv(ddx, ddy - 1, ddz)) : 0.0f;
            };
            auto GZ = [&](int ddz) -> float {
              return in_vol(0, 0, ddz) ? cdiff(Dv(0, 0, ddz + 1), Dv(0, 0, ddz - 1)) : 0.0f;
            };
            float *h = hv[u];
            h[0] = cdiff(GX(1, 0, 0), GX(-1, 0, 0));
            h[1] = cdiff(GX(0, 1, 0), GX(0, -1, 0));
            h[2] = cdiff(GX(0, 0, 1), GX(0, 0, -1));
            h[3] = cdiff(GY(0, 1, 0), GY(0, -1, 0));
            h[4] = cdiff(GY(0, 0, 1), GY(0, 0, -1));
            h[5] = cdiff(GZ(1), GZ(-1));
            const bool pd = pd_test(h[0], h[1], h[2], h[3], h[4], h[5]);
            idx[u] = zh * WH + (int64_t)Y * W + X;
            mask[S.vox + idx[u]] = pd ? 1 : 0;
            fgv[u] = pd && idx[u] != 0;
            nfg += fgv[u];
          }
        }
      }
      // warp-aggregated append to the foreground list
      const int lane = t & 31;
      int incl = nfg;
      for (int dd = 1; dd < 32; dd <<= 1) {
        const int v = __shfl_up_sync(0xFFFFFFFFu, incl, dd);
        if (lane >= dd) incl += v;
      }
      const int tot = __shfl_sync(0xFFFFFFFFu, incl, 31);
      unsigned long long base = 0;
      if (lane == 31 && tot) base = atomicAdd(&fg_count[blockIdx.y * kFgCountStride], (unsigned long long)tot);
      base = __shfl_sync(0xFFFFFFFFu, base, 31) + (unsigned long long)(incl - nfg);
      for (int u = 0; u < 2; u++) {
        if (!fgv[u]) continue;
        if ((int64_t)base < S.fg_cap) {
          FgEntry e;
          e.idx = (int32_t)idx[u];
          e.norm = __ldcg(norm + S.vox + idx[u]);
#pragma unroll
          for (int k = 0; k < 6; k++) e.h[k] = hv[u][k];
          float4 *dst = reinterpret_cast<float4 *>(fg + S.fg + base);
          const float4 *src = reinterpret_cast<const float4 *>(&e);
          dst[0] = src[0];
          dst[1] = src[1];
          fg_idx[S.fg + base] = (int32_t)idx[u];
        }
        base++;
      }
    }
  }
}

// ------------------------------------------------------------------ radius-specialised sweeps
// For common sigma pairs the chain runs as two z-sweeps with the four tap radii as
// template parameters (RA/RB: xy radius of the small/large scale, ZA/ZB: z radius):
//
//   k_dog_sweep   normalized -> DoG volume.  A block owns a kDTX x kDTY tile and sweeps
//                 z; stage A filters slice it along x (TMA-loaded, double-buffered), stage
//                 B filters slice it-1 along y and feeds the z shift register, which emits
//                 DoG slice it-1-RZ straight to global memory.  One barrier per slice.
//                 Tap pairs shared by both scales sit in per-thread registers, the taps of
//                 the wider scale alone are constant-bank operands.  The z shift
//                 register never moves: output zo lives in slot zo mod (2RZ+1), and a
//                 switch on the step's phase picks the compile-time slot of every tap.
//                 Every output is the reference's FMA chain, zero taps at the borders
//                 included, so the volume equals the separate passes bit for bit.
//   k_hess_sweep  DoG -> mask + foreground list.  A block owns a kHTX x kHTY tile; DoG slices
//                 (tile + 2-voxel halo, zero outside the volume) arrive by TMA into an
//                 8-slot ring, up to five slices ahead; each thread tests one x quad.  No
//                 block barrier per slice: warps release ring slots through mbarriers.
//                 The normalized values the list carries are read from global memory by
//                 the threads whose quad has foreground.
//
// The split costs one write and one read of the DoG volume but frees the Hessian stage
// from the z shift register's registers, so several Hessian blocks share an SM.
constexpr int kDTX = 32, kDTY = 16;     // DoG tile (three 256-thread blocks per SM, 80 registers)
constexpr int kHTX = 32, kHTY = 16;     // Hessian tile (six blocks per SM)
constexpr int kHPX = kHTX + 8;          // Hessian ring row: columns x0-4 .. x0+kHTX+3 (16-byte aligned start)
constexpr int kHPY = kHTY + 4;
constexpr int kHRing = 8;              // ring slots; a slot is 40 x 20 floats = 25 x 128 bytes
constexpr int kHThreads = kHTX / 4 * kHTY;   // one x quad per thread

// Input slices of the DoG sweep in flight: slice it + kDogIn - 1 is requested while slice it
// is filtered (2, 3 and 4 measured the same on the camera stack; 2 keeps the buffer index a
// bit mask).
#ifndef HDOG_DOG_STAGES
#define HDOG_DOG_STAGES 2
#endif
constexpr int kDogIn = HDOG_DOG_STAGES;

template <int RA, int RB, int ZA, int ZB>
struct DogT {
  static constexpr int RXY = RA > RB ? RA : RB;
  static constexpr int RZ = ZA > ZB ? ZA : ZB;
  static constexpr int WIN = 2 * RZ + 1;
  static constexpr int HX = (RXY + 3) / 4 * 4;                // x halo, 16-byte aligned
  static constexpr int BW = kDTX + 2 * HX;                    // staged input box
  static constexpr int BH = kDTY + 2 * RXY;
  static constexpr int IN_FLOATS = (BW * BH + 31) / 32 * 32;  // 128-byte multiple
  static constexpr int XQ = kDTX / 4;                         // x-pass items per row
  static constexpr int XITEMS = BH * XQ;
  static constexpr int OFF = HX - RXY;                        // item q reads from column 4q + OFF
  static constexpr int NV = (OFF + 2 * RXY + 4 + 3) / 4 * 4;  // inputs staged per item
  static constexpr int NT = kDTX * kDTY / 2;                  // 256: two z columns per thread
  static constexpr size_t SMEM = (size_t)kDogIn * IN_FLOATS * 4 + (size_t)2 * BH * kDTX * 8 + 8 * kDogIn + 64;
};

// Coefficient pairs (small, large) of the taps both scales share, |j| <= min(RA, RB),
// held in registers for the whole sweep: an f32x2 FMA takes its operands from registers,
// so pairs re-read from the constant bank would cost a load each use.  Taps of the
// wider scale alone stay constant-bank operands of scalar FMAs.
template <int RA, int RB>
struct TapPairs {
  static constexpr int RS = RA < RB ? RA : RB;
  float2 k[2 * RS + 1];
  static constexpr int N = 2 * RS + 1;
  __device__ __forceinline__ void load(const DogTaps &T, int ka, int kb) {
#pragma unroll
    for (int j = -RS; j <= RS; j++) k[j + RS] = make_float2(T.k[ka][RA - j], T.k[kb][RB - j]);
  }
  // The pairs as written by stage(): read back from shared memory, they are per-thread
  // registers, so the f32x2 FMAs use them directly instead of copying each pair out of
  // the uniform registers a kernel-parameter value would live in.
  __device__ __forceinline__ static void stage(const DogTaps &T, int ka, int kb, float2 *sh) {
#pragma unroll
    for (int j = -RS; j <= RS; j++) sh[j + RS] = make_float2(T.k[ka][RA - j], T.k[kb][RB - j]);
  }
  __device__ __forceinline__ void load_shared(const float2 *sh) {
#pragma unroll
    for (int i = 0; i < N; i++) k[i] = sh[i];
  }
};

// One tap of both scales: j is the input offset, the coefficient index r - j as in the
// reference's `sum = fma(k[r - j], s[x + j], sum)`.
template <int RA, int RB, int J>
__device__ __forceinline__ void tap2(const DogTaps &T, const TapPairs<RA, RB> &K, int ka, int kb, float2 v,
                                     float2 &acc) {
  constexpr bool a = J >= -RA && J <= RA, b = J >= -RB && J <= RB;
  if (a && b) acc = fma2(K.k[J + TapPairs<RA, RB>::RS], v, acc);
  else if (b) acc.y = __fmaf_rn(T.k[kb][RB - J], v.y, acc.y);
  else if (a) acc.x = __fmaf_rn(T.k[ka][RA - J], v.x, acc.x);
}

// x pass input by input: staged input w[I] is tap I - BASE - o of output o (o = 0..3), so its
// duplicated pair (one value for both scales of an f32x2 FMA) is formed once and used by up
// to four consecutive FMAs.  Every output still takes its taps in ascending order.
template <int RA, int RB, int BASE, int I, int NV>
struct XIn {
  __device__ __forceinline__ static void run(const DogTaps &T, const TapPairs<RA, RB> &K, const float (&w)[NV],
                                             float2 (&a)[4]) {
    if constexpr (I < NV) {
      const float2 d = make_float2(w[I], w[I]);
      tap2<RA, RB, I - BASE>(T, K, 0, 2, d, a[0]);
      tap2<RA, RB, I - BASE - 1>(T, K, 0, 2, d, a[1]);
      tap2<RA, RB, I - BASE - 2>(T, K, 0, 2, d, a[2]);
      tap2<RA, RB, I - BASE - 3>(T, K, 0, 2, d, a[3]);
      XIn<RA, RB, BASE, I + 1, NV>::run(T, K, w, a);
    }
  }
};

template <int RA, int RB, int J, int N>
struct TapLoop {
  // x pass: taps J .. J+N-1 for the four outputs of an item
  template <int NV>
  __device__ __forceinline__ static void x4(const DogTaps &T, const TapPairs<RA, RB> &K, const float (&w)[NV],
                                            int base, float2 (&a)[4]) {
    if constexpr (N > 0) {
#pragma unroll
      for (int o = 0; o < 4; o++) {
        const float x = w[base + o + J];
        tap2<RA, RB, J>(T, K, 0, 2, make_float2(x, x), a[o]);
      }
      TapLoop<RA, RB, J + 1, N - 1>::x4(T, K, w, base, a);
    }
  }
  // y pass of rows cy (g0) and cy + 1 (g1): input row i is tap i - R of g0 and tap
  // i - R - 1 of g1, loaded once, in ascending tap order for both
  template <int STRIDE>
  __device__ __forceinline__ static void y2(const DogTaps &T, const TapPairs<RA, RB> &K, const float2 *col,
                                            float2 &g0, float2 &g1) {
    if constexpr (N > 0) {
      constexpr int R = RA > RB ? RA : RB;
      const float2 v = col[(J + R) * STRIDE];
      tap2<RA, RB, J>(T, K, 0, 2, v, g0);
      if constexpr (J > -R) tap2<RA, RB, J - 1>(T, K, 0, 2, v, g1);
      if constexpr (N == 1) tap2<RA, RB, J>(T, K, 0, 2, col[(J + R + 1) * STRIDE], g1);
      TapLoop<RA, RB, J + 1, N - 1>::template y2<STRIDE>(T, K, col, g0, g1);
    }
  }
};

// z step of phase P = zy mod WIN: input slice zy is tap d of output zo = zy - d, which
// lives in slot (zo mod WIN); then output zy - RZ is complete and its slot is cleared for
// output zy - RZ + WIN.
template <class C, int ZA, int ZB, int P, int D0, int N>
struct ZTaps {
  __device__ __forceinline__ static void run(const DogTaps &T, const TapPairs<ZA, ZB> &K, float2 (&a0)[C::WIN],
                                             float2 (&a1)[C::WIN], float2 g0, float2 g1) {
    if constexpr (N > 0) {
      constexpr int s = ((P - D0) % C::WIN + C::WIN) % C::WIN;
      tap2<ZA, ZB, D0>(T, K, 1, 3, g0, a0[s]);
      tap2<ZA, ZB, D0>(T, K, 1, 3, g1, a1[s]);
      ZTaps<C, ZA, ZB, P, D0 + 1, N - 1>::run(T, K, a0, a1, g0, g1);
    }
  }
};

template <class C, int ZA, int ZB, int P>
__device__ __forceinline__ void z_step(const DogTaps &T, const TapPairs<ZA, ZB> &K, float2 (&a0)[C::WIN],
                                       float2 (&a1)[C::WIN], float2 g0, float2 g1, float &d0, float &d1) {
  ZTaps<C, ZA, ZB, P, -C::RZ, C::WIN>::run(T, K, a0, a1, g0, g1);
  constexpr int se = ((P - C::RZ) % C::WIN + C::WIN) % C::WIN;
  d0 = __fmul_rn(__fsub_rn(a0[se].x, a0[se].y), T.normalizer);
  d1 = __fmul_rn(__fsub_rn(a1[se].x, a1[se].y), T.normalizer);
  a0[se] = make_float2(0.f, 0.f);
  a1[se] = make_float2(0.f, 0.f);
}

// Calls f(base + P, integral_constant<P>) for P = 0 .. N-1 while base + P < limit (the
// bound is uniform over the block, so every thread runs the same steps).
template <int P, int N, class F>
__device__ __forceinline__ void unroll_steps_from(F &f, int base, int limit) {
  if constexpr (P < N) {
    if (base + P < limit) {
      f(base + P, std::integral_constant<int, P>{});
      unroll_steps_from<P + 1, N>(f, base, limit);
    }
  }
}
template <int N, class F>
__device__ __forceinline__ void unroll_steps(F &f, int base, int limit) {
  unroll_steps_from<0, N>(f, base, limit);
}

// PERSIST: a grid of a few blocks per SM takes (substack, tile) items from the device work
// queue `q` until it is empty; otherwise one block per tile (blockIdx.x) and substack
// (blockIdx.y).  Results are the same either way.
template <int RA, int RB, int ZA, int ZB, bool PERSIST>
__global__ void __launch_bounds__(DogT<RA, RB, ZA, ZB>::NT, 3)
    k_dog_sweep(const __grid_constant__ CUtensorMap map, const __grid_constant__ DogTaps T, const Sub *subs,
                float *dog, int *status, WorkQueue q) {
  using C = DogT<RA, RB, ZA, ZB>;
  extern __shared__ __align__(128) unsigned char smem[];
  float *inb = reinterpret_cast<float *>(smem);
  float2 *xb = reinterpret_cast<float2 *>(smem + (size_t)kDogIn * C::IN_FLOATS * 4);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + (size_t)kDogIn * C::IN_FLOATS * 4 + (size_t)2 * C::BH * kDTX * 8);
  const int t = threadIdx.x;
  __shared__ float2 tap_sh[TapPairs<RA, RB>::N + TapPairs<ZA, ZB>::N];
  __shared__ int s_item;
  if (t == 0) {
    for (int i = 0; i < kDogIn; i++) mbar_init(&bar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    TapPairs<RA, RB>::stage(T, 0, 2, tap_sh);
    TapPairs<ZA, ZB>::stage(T, 1, 3, tap_sh + TapPairs<RA, RB>::N);
  }
  bool ok = true;
  // slices loaded by this block before the current tile: slice `it` of a tile is the block's
  // (gbase + it)-th, which picks its input buffer (g mod kDogIn) and barrier phase
  uint32_t gbase = 0;
  for (;;) {
  int sub, tile;
  __syncthreads();   // the previous tile is done with both input buffers
  if (PERSIST) {
    if (t == 0) s_item = (int)atomicAdd(q.next, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= q.total) break;
    sub = item / q.tiles;
    tile = item % q.tiles;
  } else {
    sub = blockIdx.y;
    tile = blockIdx.x;
  }
  const Sub S = subs[sub];
  const int ntx = (S.W + kDTX - 1) / kDTX, nty = (S.H + kDTY - 1) / kDTY;
  if (tile >= ntx * nty) {
    if (PERSIST) continue;
    break;
  }
  const int x0 = (tile % ntx) * kDTX, y0 = (tile / ntx) * kDTY;
  const int D = S.D, W = S.W, H = S.H;
  constexpr uint32_t tma_bytes = (uint32_t)(C::BW * C::BH * 4);
  const int tx = x0 - C::HX, ty = y0 - C::RXY;
  if (t == 0 && ok)
    for (int z = 0; z < kDogIn - 1 && z < D; z++) {
      const uint32_t g = gbase + (uint32_t)z;
      tma_slice(&map, inb + (g % kDogIn) * C::IN_FLOATS, &bar[g % kDogIn], tx, ty, z, sub, tma_bytes);
    }
  // stage B ownership: columns (cx, cy) and (cx, cy + 1) of the tile
  const int cx = t % kDTX, cy = 2 * (t / kDTX);
  const int gx = x0 + cx, gy = y0 + cy;
  const bool w0 = gx < W && gy < H, w1 = gx < W && gy + 1 < H;
  float *out0 = dog + S.vox + (int64_t)gy * W + gx;
  const int64_t WH = (int64_t)W * H;
  float2 acc0[C::WIN], acc1[C::WIN];
#pragma unroll
  for (int s = 0; s < C::WIN; s++) { acc0[s] = make_float2(0.f, 0.f); acc1[s] = make_float2(0.f, 0.f); }
  TapPairs<RA, RB> kxy;
  TapPairs<ZA, ZB> kz;
  kxy.load_shared(tap_sh);
  kz.load_shared(tap_sh + TapPairs<RA, RB>::N);
  const int nit = D + C::RZ + 1;
  // One slice step; PC is the step's position inside a group of WIN steps, so the z phase
  // of slice zy = it - 1 is the compile-time (PC - 1) mod WIN and every shift-register slot
  // is a fixed register (the loop below runs WIN steps per trip).
  auto step = [&](int it, auto PC) {
    constexpr int PH = (decltype(PC)::value + C::WIN - 1) % C::WIN;
    // slice it + kDogIn - 1 goes to the buffer of slice it - 1, read before the last barrier
    const uint32_t gn = gbase + (uint32_t)(it + kDogIn - 1);
    if (t == 0 && ok && it + kDogIn - 1 < D)
      tma_slice(&map, inb + (gn % kDogIn) * C::IN_FLOATS, &bar[gn % kDogIn], tx, ty, it + kDogIn - 1, sub, tma_bytes);
    // ---- B: y pass of slice zy (zero past the volume: the border taps still multiply),
    // z shift register, DoG slice zy - RZ
    const int zy = it - 1;
    if (zy >= 0) {
      float2 g0 = make_float2(0.f, 0.f), g1 = make_float2(0.f, 0.f);
      if (zy < D)
        TapLoop<RA, RB, -C::RXY, 2 * C::RXY + 1>::template y2<kDTX>(
            T, kxy, xb + (zy & 1) * C::BH * kDTX + cy * kDTX + cx, g0, g1);
      float d0, d1;
      z_step<C, ZA, ZB, PH>(T, kz, acc0, acc1, g0, g1, d0, d1);
      const int zo = zy - C::RZ;
      if (zo >= 0) {
        if (w0) out0[zo * WH] = d0;
        if (w1) out0[zo * WH + W] = d1;
      }
    }
    // ---- A: x pass of slice it
    if (it < D) {
      const uint32_t gi = gbase + (uint32_t)it;
      if (ok && !mbar_wait(&bar[gi % kDogIn], (gi / kDogIn) & 1)) {
        ok = false;
        atomicExch(status, HDOG_ERR_TIMEOUT);
      }
      const float *ib = inb + (gi % kDogIn) * C::IN_FLOATS;
      float2 *xo = xb + (it & 1) * C::BH * kDTX;
      // one item per thread when the items fit the block (no loop, no reconvergence)
      for (int item = t; item < C::XITEMS; item += (C::XITEMS <= C::NT ? C::XITEMS : C::NT)) {
        const int row = item / C::XQ, q = item % C::XQ;
        const float *in = ib + row * C::BW + 4 * q;
        float w[C::NV];
#pragma unroll
        for (int i = 0; i < C::NV; i += 4) {
          const float4 f = *reinterpret_cast<const float4 *>(in + i);
          w[i] = f.x; w[i + 1] = f.y; w[i + 2] = f.z; w[i + 3] = f.w;
        }
        float2 a[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        XIn<RA, RB, C::OFF + C::RXY, 0, C::NV>::run(T, kxy, w, a);
        float4 *o = reinterpret_cast<float4 *>(xo + row * kDTX + 4 * q);
        o[0] = make_float4(a[0].x, a[0].y, a[1].x, a[1].y);
        o[1] = make_float4(a[2].x, a[2].y, a[3].x, a[3].y);
      }
    }
    __syncthreads();
  };
  for (int base = 0; base < nit; base += C::WIN)
    unroll_steps<C::WIN>(step, base, nit);
  gbase += (uint32_t)D;
  if (!PERSIST) break;
  }
}

// Central difference of the Hessian stage.  The reference writes ((0 + a) - b) * 0.5; the
// `0 +` only turns -0 into +0, and a zero's sign never changes a magnitude, a comparison
// or a fixed-point sum, so the mask and every record stay identical without it.
__device__ __forceinline__ float hdiff(float plus, float minus) { return __fmul_rn(__fsub_rn(plus, minus), 0.5f); }
// The same on two voxels at once (each lane rounds as the scalar operations do).
__device__ __forceinline__ float2 hd2(float2 plus, float2 minus) {
  return mul2(sub2(plus, minus), make_float2(0.5f, 0.5f));
}

// The pinned Sylvester test (common.cuh pd_test) on two voxels: every product and FMA is
// the scalar one lane by lane; fma(-(a*b), c, t) is written fma(a*b, c * -1, t), the same
// exact product with the sign moved.  Returns the two results in bits 0 and 8.
__device__ __forceinline__ uint32_t pd_test2(float2 xx, float2 xy, float2 xz, float2 yy, float2 yz, float2 zz) {
  const float2 m1 = make_float2(-1.0f, -1.0f);
  const float2 p = mul2(xx, yy);
  const float2 q = mul2(mul2(make_float2(2.0f, 2.0f), xy), yz);
  float2 t = fma2(p, zz, mul2(q, xz));
  t = fma2(mul2(xx, yz), mul2(yz, m1), t);
  t = fma2(mul2(yy, xz), mul2(xz, m1), t);
  const float2 xy2 = mul2(xy, xy);
  const float2 rhs = mul2(mul2(zz, xy), xy);
  const uint32_t a = (xx.x < 0.0f) & (p.x > xy2.x) & (t.x < rhs.x);
  const uint32_t b = (xx.y < 0.0f) & (p.y > xy2.y) & (t.y < rhs.y);
  return a | (b << 8);
}

// Gradient pairs of one ring row.  Voxel pairs come in two frames: the C frame
// (X0, X0+1), (X0+2, X0+3) -- the thread's own quad -- and the G frame (X0-1, X0),
// (X0+1, X0+2), (X0+3, X0+4), in which x differences of pairs loaded on 8-byte
// boundaries land without repacking.  gx in the G frame from the row's columns
// X0-2 .. X0+5 (l = X0-2, X0-1; c = the quad; r = X0+4, X0+5).
__device__ __forceinline__ void gx_g(float2 l, float2 c0, float2 c1, float2 r, float2 (&g)[3]) {
  g[0] = hd2(c0, l);
  g[1] = hd2(c1, c0);
  g[2] = hd2(r, c1);
}

__device__ __forceinline__ void ld_row(const float *p, float2 &l, float2 &c0, float2 &c1, float2 &r) {
  l = *reinterpret_cast<const float2 *>(p - 2);
  const float4 c = *reinterpret_cast<const float4 *>(p);
  c0 = make_float2(c.x, c.y);
  c1 = make_float2(c.z, c.w);
  r = *reinterpret_cast<const float2 *>(p + 4);
}
__device__ __forceinline__ void ld_quad(const float *p, float2 &c0, float2 &c1) {
  const float4 c = *reinterpret_cast<const float4 *>(p);
  c0 = make_float2(c.x, c.y);
  c1 = make_float2(c.z, c.w);
}

// Staged list entries per warp: one iteration adds at most 128 (four voxels per lane).
constexpr int kHStage = 128;

// Moves a warp's `n` staged entries to the substack's list: one slot reservation, then
// each lane completes whole entries -- the normalized value at the entry's voxel is
// gathered here, once per flush rather than on every slice -- and stores them as
// consecutive 32-byte entries.  Entries past the list's capacity are dropped but counted,
// so the host sees the overflow and redoes the batch.
__device__ __forceinline__ void flush_stage(const FgEntry *stage, int n, const Sub &S, const float *norm, FgEntry *fg,
                                            int32_t *fg_idx, unsigned long long *count) {
  __syncwarp();
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(count, (unsigned long long)n);
  base = __shfl_sync(0xFFFFFFFFu, base, 0);
  const int64_t room = S.fg_cap - (int64_t)base;
  const int keep = room <= 0 ? 0 : (room < n ? (int)room : n);
  const float *nv = norm + S.vox;
  // every lane's gathers are issued before any of them is used, so a flush waits for one
  // global-load latency rather than one per entry
  constexpr int kPer = kHStage / 32;
  int32_t idx[kPer];
  float nvv[kPer];
#pragma unroll
  for (int u = 0; u < kPer; u++) {
    const int i = lane + 32 * u;
    idx[u] = i < keep ? stage[i].idx : 0;
    nvv[u] = i < keep ? __ldg(nv + idx[u]) : 0.0f;
  }
#pragma unroll
  for (int u = 0; u < kPer; u++) {
    const int i = lane + 32 * u;
    if (i < keep) {
      const float4 *src = reinterpret_cast<const float4 *>(stage + i);
      float4 a = src[0];
      a.y = nvv[u];
      float4 *dst = reinterpret_cast<float4 *>(fg + S.fg + base + i);
      dst[0] = a;
      dst[1] = src[1];
      fg_idx[S.fg + base + i] = idx[u];
    }
  }
  __syncwarp();
}

// Blocks per SM the Hessian sweep is compiled for: five fit its z pipeline in 96
// registers without spilling.
#ifndef HDOG_HESS_BLOCKS
#define HDOG_HESS_BLOCKS 5
#endif
// PERSIST: a grid of a few blocks per SM takes (substack, tile) items from the device work
// queue `q` until it is empty; otherwise one block per tile (blockIdx.x) and substack
// (blockIdx.y).  Results are the same either way.
template <bool PERSIST>
__global__ void __launch_bounds__(kHThreads, HDOG_HESS_BLOCKS)
    k_hess_sweep(const __grid_constant__ CUtensorMap map, const Sub *subs, const float *norm, uint8_t *mask,
                 FgEntry *fg, int32_t *fg_idx, unsigned long long *fg_count, int *status, WorkQueue q) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int PL = kHPX * kHPY;
  constexpr uint32_t tma_bytes = (uint32_t)(PL * 4);
  float *ring = reinterpret_cast<float *>(smem);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + (size_t)kHRing * PL * 4);
  // done[i % kHRing] completes when every warp has finished the block's i-th iteration, with
  // its last reads of that iteration's DoG slice zh-2
  uint64_t *done = bar + kHRing;
  const int t = threadIdx.x;
  // this warp's staging of list entries (flushed to the global list kHStage at a time at most)
  FgEntry *stage = reinterpret_cast<FgEntry *>(smem + (size_t)kHRing * PL * 4 + 2 * kHRing * 8) + (t >> 5) * kHStage;
  __shared__ int s_item;
  if (t == 0) {
    for (int i = 0; i < kHRing; i++) mbar_init(&bar[i], 1);
    for (int i = 0; i < kHRing; i++) mbar_init(&done[i], kHThreads / 32);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  bool ok = true;
  // slices loaded into the ring and iterations run by this block before the current tile:
  // every tile loads its slices -2 .. D+1 once and runs D iterations, so the barrier phases
  // continue from tile to tile
  uint32_t zbase = 0, ibase = 0;
  for (;;) {
  int sub, tile;
  __syncthreads();   // every warp is done with the previous tile's ring slots
  if (PERSIST) {
    if (t == 0) s_item = (int)atomicAdd(q.next, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= q.total) break;
    sub = item / q.tiles;
    tile = item % q.tiles;
  } else {
    sub = blockIdx.y;
    tile = blockIdx.x;
  }
  const Sub S = subs[sub];
  const int ntx = (S.W + kHTX - 1) / kHTX, nty = (S.H + kHTY - 1) / kHTY;
  if (tile >= ntx * nty) {
    if (PERSIST) continue;
    break;
  }
  const int x0 = (tile % ntx) * kHTX, y0 = (tile / ntx) * kHTY;
  int staged = 0;   // entries in this warp's staging buffer (the same in every lane)
  const int D = S.D, W = S.W, H = S.H;
  const int32_t WH = W * H;
  const int tx = x0 - 4, ty = y0 - 2;
  // ring slot of DoG slice z (z = -2 .. D+1; slices outside the volume arrive zero-filled)
  auto slot = [zbase](int z) { return (int)((zbase + (uint32_t)(z + 2)) % kHRing); };
  // use k of slot s (k-th slice loaded into it) completes barrier phase k & 1
  auto use = [zbase](int z) { return (int)((zbase + (uint32_t)(z + 2)) / kHRing); };
  // slices -2 .. 4 up front, then slice zh + 5 while slice zh is tested: the slot it
  // reuses held slice zh - 3, last read one barrier earlier
  if (t == 0 && ok)
    for (int z = -2; z <= 4 && z <= D + 1; z++)
      tma_slice(&map, ring + slot(z) * PL, &bar[slot(z)], tx, ty, z, sub, tma_bytes);
  for (int z = -2; z <= 1; z++)
    if (ok && !mbar_wait(&bar[slot(z)], use(z) & 1)) {
      ok = false;
      atomicExch(status, HDOG_ERR_TIMEOUT);
    }
  const int q = t % (kHTX / 4), ly = t / (kHTX / 4);
  const int X0 = x0 + 4 * q, Y = y0 + ly;
  const int b = (ly + 2) * kHPX + 4 * q + 4;   // ring index of column X0 on row Y
  // every in-plane gradient position of the quad inside the volume: the z-pipelined
  // stencil below (only the z neighbours can fall outside); the frame's edges take the
  // literal zero-halo path voxel by voxel.  Fixed per thread for the whole sweep.
  const bool interior = X0 >= 1 && X0 + 3 <= W - 2 && Y >= 1 && Y <= H - 2;
  // z pipeline of the interior path: first derivatives of slices zh-1 and zh on row Y
  // (gx in the G frame, gy and gz in the C frame) and DoG of slices zh and zh+1 on row Y
  const float2 zero2 = make_float2(0.0f, 0.0f);
  float2 gxm[3] = {zero2, zero2, zero2}, gx0[3];
  float2 gym[2] = {zero2, zero2}, gy0[2], gzm[2] = {zero2, zero2}, gz0[2];
  float2 fm[2] = {zero2, zero2}, f0[2];
  if (interior) {
    // slice 0: gx, gy on row Y; gz from slices 1 and -1 (zero)
    const float *P0 = ring + slot(0) * PL + b, *P1 = ring + slot(1) * PL + b;
    float2 l, r, u0, u1, d0, d1;
    ld_row(P0, l, f0[0], f0[1], r);
    gx_g(l, f0[0], f0[1], r, gx0);
    ld_quad(P0 - kHPX, u0, u1);
    ld_quad(P0 + kHPX, d0, d1);
    gy0[0] = hd2(d0, u0);
    gy0[1] = hd2(d1, u1);
    float2 p0, p1;
    ld_quad(P1, p0, p1);
    gz0[0] = hd2(p0, zero2);
    gz0[1] = hd2(p1, zero2);
    fm[0] = f0[0]; fm[1] = f0[1];
    f0[0] = p0; f0[1] = p1;
  }
  for (int zh = 0; zh < D; zh++) {
    // DoG slice zh+5 reuses the slot of slice zh-3, read for the last time in iteration
    // zh-1: the producer waits until every warp is past it (warps otherwise run up to the
    // ring's depth apart)
    if (t == 0 && ok && zh + 5 <= D + 1) {
      const uint32_t prev = ibase + (uint32_t)zh - 1u;
      if (zh >= 1 && !mbar_wait(&done[prev % kHRing], (prev / kHRing) & 1)) {
        ok = false;
        atomicExch(status, HDOG_ERR_TIMEOUT);
      }
      if (ok) tma_slice(&map, ring + slot(zh + 5) * PL, &bar[slot(zh + 5)], tx, ty, zh + 5, sub, tma_bytes);
    }
    // slices zh-2 .. zh+1 were waited for already; zh+2 is new
    if (ok && !mbar_wait(&bar[slot(zh + 2)], use(zh + 2) & 1)) {
      ok = false;
      atomicExch(status, HDOG_ERR_TIMEOUT);
    }
    uint32_t mword = 0;
    const int32_t i0 = zh * WH + Y * W + X0;
    float hv[4][6];
    if (interior) {
      const float *P0 = ring + slot(zh) * PL + b, *P1 = ring + slot(zh + 1) * PL + b;
      const float *P2 = ring + slot(zh + 2) * PL + b;
      // ---- in-plane second derivatives of slice zh
      float2 hxx[2], hxy[3], hyy[2];
      hxx[0] = hd2(gx0[1], gx0[0]);
      hxx[1] = hd2(gx0[2], gx0[1]);
      {
        float2 l, c0, c1, r, gu[3], gd[3];
        ld_row(P0 - kHPX, l, c0, c1, r);
        gx_g(l, c0, c1, r, gu);
        float2 e0, e1;
        ld_quad(P0 - 2 * kHPX, e0, e1);
        const float2 gyu0 = hd2(fm[0], e0), gyu1 = hd2(fm[1], e1);   // gy on row Y-1
        ld_row(P0 + kHPX, l, c0, c1, r);
        gx_g(l, c0, c1, r, gd);
        ld_quad(P0 + 2 * kHPX, e0, e1);
        const float2 gyd0 = hd2(e0, fm[0]), gyd1 = hd2(e1, fm[1]);                      // gy on row Y+1
#pragma unroll
        for (int i = 0; i < 3; i++) hxy[i] = hd2(gd[i], gu[i]);
        hyy[0] = hd2(gyd0, gyu0);
        hyy[1] = hd2(gyd1, gyu1);
      }
      // ---- first derivatives of slice zh+1 on row Y, then the z second derivatives
      float2 gxp[3], gyp[2], gzp[2], fp[2];
      {
        float2 l, r, u0, u1, d0, d1;
        l = *reinterpret_cast<const float2 *>(P1 - 2);
        r = *reinterpret_cast<const float2 *>(P1 + 4);
        gx_g(l, f0[0], f0[1], r, gxp);
        ld_quad(P1 - kHPX, u0, u1);
        ld_quad(P1 + kHPX, d0, d1);
        gyp[0] = hd2(d0, u0);
        gyp[1] = hd2(d1, u1);
        ld_quad(P2, fp[0], fp[1]);
        const bool zin = zh + 1 < D;   // gz outside the volume is zero
        gzp[0] = zin ? hd2(fp[0], fm[0]) : zero2;
        gzp[1] = zin ? hd2(fp[1], fm[1]) : zero2;
      }
      float2 hxz[3], hyz[2], hzz[2];
#pragma unroll
      for (int i = 0; i < 3; i++) hxz[i] = hd2(gxp[i], gxm[i]);
      hyz[0] = hd2(gyp[0], gym[0]);
      hyz[1] = hd2(gyp[1], gym[1]);
      hzz[0] = hd2(gzp[0], gzm[0]);
      hzz[1] = hd2(gzp[1], gzm[1]);
      // advance the pipeline
#pragma unroll
      for (int i = 0; i < 3; i++) { gxm[i] = gx0[i]; gx0[i] = gxp[i]; }
#pragma unroll
      for (int j = 0; j < 2; j++) {
        gym[j] = gy0[j]; gy0[j] = gyp[j];
        gzm[j] = gz0[j]; gz0[j] = gzp[j];
        fm[j] = f0[j]; f0[j] = fp[j];
      }
      // G frame -> C frame for the two elements that live there (voxel 2j+h)
      const float2 cxy[2] = {make_float2(hxy[0].y, hxy[1].x), make_float2(hxy[1].y, hxy[2].x)};
      const float2 cxz[2] = {make_float2(hxz[0].y, hxz[1].x), make_float2(hxz[1].y, hxz[2].x)};
#pragma unroll
      for (int j = 0; j < 2; j++) {
        mword |= pd_test2(hxx[j], cxy[j], cxz[j], hyy[j], hyz[j], hzz[j]) << (16 * j);
        hv[2 * j][0] = hxx[j].x; hv[2 * j + 1][0] = hxx[j].y;
        hv[2 * j][1] = cxy[j].x; hv[2 * j + 1][1] = cxy[j].y;
        hv[2 * j][2] = cxz[j].x; hv[2 * j + 1][2] = cxz[j].y;
        hv[2 * j][3] = hyy[j].x; hv[2 * j + 1][3] = hyy[j].y;
        hv[2 * j][4] = hyz[j].x; hv[2 * j + 1][4] = hyz[j].y;
        hv[2 * j][5] = hzz[j].x; hv[2 * j + 1][5] = hzz[j].y;
      }
      *reinterpret_cast<uint32_t *>(mask + S.vox + i0) = mword;
    } else {
#pragma unroll
      for (int o = 0; o < 4; o++) {
        const int X = X0 + o;
        if (X >= W || Y >= H) continue;
        const int ex = 4 * q + o + 4, ey = ly + 2;
        auto Dv = [&](int ddx, int ddy, int ddz) -> float {
          return ring[slot(zh + ddz) * PL + (ey + ddy) * kHPX + (ex + ddx)];
        };
        auto in_vol = [&](int ddx, int ddy, int ddz) -> bool {
          const int xx = X + ddx, yy = Y + ddy, zz = zh + ddz;
          return xx >= 0 && xx < W && yy >= 0 && yy < H && zz >= 0 && zz < D;
        };
        auto GX = [&](int ddx, int ddy, int ddz) -> float {
          return in_vol(ddx, ddy, ddz) ? hdiff(Dv(ddx + 1, ddy, ddz), Dv(ddx - 1, ddy, ddz)) : 0.0f;
        };
        auto GY = [&](int ddx, int ddy, int ddz) -> float {
          return in_vol(ddx, ddy, ddz) ? hdiff(Dv(ddx, ddy + 1, ddz), Dv(ddx, ddy - 1, ddz)) : 0.0f;
        };
        auto GZ = [&](int ddz) -> float {
          return in_vol(0, 0, ddz) ? hdiff(Dv(0, 0, ddz + 1), Dv(0, 0, ddz - 1)) : 0.0f;
        };
        hv[o][0] = hdiff(GX(1, 0, 0), GX(-1, 0, 0));
        hv[o][1] = hdiff(GX(0, 1, 0), GX(0, -1, 0));
        hv[o][2] = hdiff(GX(0, 0, 1), GX(0, 0, -1));
        hv[o][3] = hdiff(GY(0, 1, 0), GY(0, -1, 0));
        hv[o][4] = hdiff(GY(0, 0, 1), GY(0, 0, -1));
        hv[o][5] = hdiff(GZ(1), GZ(-1));
        const bool pdv = pd_test(hv[o][0], hv[o][1], hv[o][2], hv[o][3], hv[o][4], hv[o][5]);
        mask[S.vox + i0 + o] = pdv ? 1 : 0;
        // voxel 0 is background (its label is 0 in the reference's CCL)
        mword |= (pdv && i0 + o != 0 ? 1u : 0u) << (8 * o);
      }
    }
    // the foreground voxels go to the warp's staging buffer in shared memory; a full buffer
    // goes to the global list with one slot reservation and coalesced stores (and the
    // entries' normalized values).  Warps without foreground skip all of it; each lane's
    // place comes from three bit-sliced ballots of its count.
    const int nfg = __popc(mword);
    const unsigned any = __ballot_sync(0xFFFFFFFFu, nfg != 0);
    if (any) {
      const int lane = t & 31;
      const unsigned b0 = __ballot_sync(0xFFFFFFFFu, nfg & 1), b1 = __ballot_sync(0xFFFFFFFFu, nfg & 2),
                     b2 = __ballot_sync(0xFFFFFFFFu, nfg & 4);
      const unsigned lt = (1u << lane) - 1u;
      const int excl = __popc(b0 & lt) + 2 * __popc(b1 & lt) + 4 * __popc(b2 & lt);
      const int tot = __popc(b0) + 2 * __popc(b1) + 4 * __popc(b2);
      if (staged + tot > kHStage) {
        flush_stage(stage, staged, S, norm, fg, fg_idx, &fg_count[sub * kFgCountStride]);
        staged = 0;
      }
      int k = staged + excl;
#pragma unroll
      for (int o = 0; o < 4; o++) {
        if (!((mword >> (8 * o)) & 1u)) continue;
        float4 *dst = reinterpret_cast<float4 *>(stage + k);
        dst[0] = make_float4(__int_as_float(i0 + o), 0.0f, hv[o][0], hv[o][1]);
        dst[1] = make_float4(hv[o][2], hv[o][3], hv[o][4], hv[o][5]);
        k++;
      }
      staged += tot;
    }
    __syncwarp();
    if ((t & 31) == 0) mbar_arrive(&done[(ibase + (uint32_t)zh) % kHRing]);
  }
  if (staged) flush_stage(stage, staged, S, norm, fg, fg_idx, &fg_count[sub * kFgCountStride]);
  zbase += (uint32_t)(D + 4);
  ibase += (uint32_t)D;
  if (!PERSIST) break;
  }
}

// ------------------------------------------------------------------ host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// Radius-specialised instantiations: (small xy, large xy, small z, large z) tap radii.
// (4, 6, 3, 5): sigma (2.0, 1.5) / (3.2, 2.4); (8, 12, 4, 5): sigma (4.0, 1.8) / (6.0, 2.7).
typedef void (*DogSweepKernel)(CUtensorMap, DogTaps, const Sub *, float *, int *, WorkQueue);
struct SweepInst {
  int ra, rb, za, zb;
  DogSweepKernel fn, fn_persist;
  size_t smem;
  int threads, bw, bh, hx, rxy;
};
template <int RA, int RB, int ZA, int ZB>
constexpr SweepInst sweep_inst() {
  using C = DogT<RA, RB, ZA, ZB>;
  return SweepInst{RA, RB, ZA, ZB, k_dog_sweep<RA, RB, ZA, ZB, false>, k_dog_sweep<RA, RB, ZA, ZB, true>,
                   C::SMEM, C::NT, C::BW, C::BH, C::HX, C::RXY};
}
static const SweepInst kSweepInst[] = {sweep_inst<4, 6, 3, 5>(), sweep_inst<8, 12, 4, 5>()};

static const SweepInst *find_inst(const DogTaps &T) {
  for (const SweepInst &s : kSweepInst)
    if (s.ra == T.r[0] && s.rb == T.r[2] && s.za == T.r[1] && s.zb == T.r[3]) return &s;
  return nullptr;
}

static constexpr size_t kHessSmem =
    (size_t)kHRing * kHPX * kHPY * 4 + (2 * kHRing) * 8 + (size_t)(kHThreads / 32) * kHStage * sizeof(FgEntry);
static_assert((kHPX * kHPY * 4) % 128 == 0, "TMA ring slots must start on 128-byte boundaries");

// Whether the fused sweep handles these parameters (else the separate passes run).
bool sweep_supported(const DogTaps &T, int W, int max_smem) {
  if (W % 4 != 0 || encode_fn() == nullptr) return false;
  const SweepInst *si = find_inst(T);
  if (si) return (int)si->smem <= max_smem && (int)kHessSmem <= max_smem;
  const int rxy = max(T.r[0], T.r[2]), rz = max(T.r[1], T.r[3]);
  if (rxy > kMaxSweepRxy || rz > 8) return false;
  return (int)sweep_smem_bytes(rxy) <= max_smem;
}

static CUresult encode_map(CUtensorMap *map, const float *base, int W, int H, int D, int nsub, int bw, int bh) {
  const cuuint64_t dims[4] = {(cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D, (cuuint64_t)nsub};
  const cuuint64_t strides[3] = {(cuuint64_t)W * 4, (cuuint64_t)W * H * 4, (cuuint64_t)W * H * D * 4};
  const cuuint32_t box[4] = {(cuuint32_t)bw, (cuuint32_t)bh, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float *>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
}

// One launch of a radius-specialised DoG sweep: a block per tile and substack, or (per_sm > 0)
// per_sm blocks per SM over the work queue whose counter is *qctr (zeroed here first).
static void dog_sweep_launch(const SweepInst *si, const CUtensorMap &map_n, const DogTaps &T, const Sub *d_subs,
                             int nsub, int W, int H, float *dog, int *d_status, const LaunchShape &ls,
                             unsigned *qctr, cudaStream_t s) {
  const unsigned tiles_d = ceil_div(W, kDTX) * ceil_div(H, kDTY);
  if (ls.dog_per_sm > 0 && qctr) {
    zero_async(qctr, sizeof(unsigned), s);
    const WorkQueue q{qctr, (int)(tiles_d * (unsigned)nsub), (int)tiles_d};
    const unsigned grid = std::min<unsigned>((unsigned)(ls.dog_per_sm * ls.num_sms), tiles_d * (unsigned)nsub);
    cudaFuncSetAttribute(si->fn_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)si->smem);
    KLAUNCH("k_dog_sweep", s, (si->fn_persist<<<grid, si->threads, si->smem, s>>>(map_n, T, d_subs, dog, d_status, q)));
    return;
  }
  cudaFuncSetAttribute(si->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)si->smem);
  KLAUNCH("k_dog_sweep", s, (si->fn<<<dim3(tiles_d, nsub), si->threads, si->smem, s>>>(map_n, T, d_subs, dog, d_status,
                                                                                        WorkQueue{})));
}

bool launch_dog_sweep(const Sub *d_subs, int nsub, int W, int H, int D, const DogTaps &T, const float *norm,
                      float *dog, int *d_status, int max_smem, cudaStream_t s) {
  const SweepInst *si = find_inst(T);
  if (!si || W % 4 != 0 || (int)si->smem > max_smem || encode_fn() == nullptr) return false;
  if ((reinterpret_cast<uintptr_t>(norm) & 15) != 0) return false;
  CUtensorMap map_n;
  if (encode_map(&map_n, norm, W, H, D, nsub, si->bw, si->bh) != CUDA_SUCCESS) return false;
  dog_sweep_launch(si, map_n, T, d_subs, nsub, W, H, dog, d_status, LaunchShape{}, nullptr, s);
  return true;
}

int launch_dog_hess(const Sub *d_subs, int nsub, int W, int H, int D, const DogTaps &T, const float *norm,
                    float *dog, uint8_t *mask, FgEntry *fg, int32_t *fg_idx, unsigned long long *fg_count,
                    int *d_status, const LaunchShape &ls, unsigned *qctr, cudaStream_t s) {
  const int rxy = max(T.r[0], T.r[2]), rz = max(T.r[1], T.r[3]);
  zero_async(fg_count, (size_t)nsub * kFgCountStride * sizeof(unsigned long long), s);
  const SweepInst *si = find_inst(T);
  if (si) {
    CUtensorMap map_n, map_d;
    if (encode_map(&map_n, norm, W, H, D, nsub, si->bw, si->bh) != CUDA_SUCCESS) return -1;
    if (encode_map(&map_d, dog, W, H, D, nsub, kHPX, kHPY) != CUDA_SUCCESS) return -1;
    dog_sweep_launch(si, map_n, T, d_subs, nsub, W, H, dog, d_status, ls, qctr, s);
    const unsigned tiles_h = ceil_div(W, kHTX) * ceil_div(H, kHTY);
    if (ls.hess_per_sm > 0 && qctr) {
      zero_async(qctr + 1, sizeof(unsigned), s);
      const WorkQueue q{qctr + 1, (int)(tiles_h * (unsigned)nsub), (int)tiles_h};
      const unsigned grid = std::min<unsigned>((unsigned)(ls.hess_per_sm * ls.num_sms), tiles_h * (unsigned)nsub);
      cudaFuncSetAttribute(k_hess_sweep<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kHessSmem);
      KLAUNCH("k_hess_sweep", s, (k_hess_sweep<true><<<grid, kHThreads, kHessSmem, s>>>(
                                     map_d, d_subs, norm, mask, fg, fg_idx, fg_count, d_status, q)));
    } else {
      cudaFuncSetAttribute(k_hess_sweep<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kHessSmem);
      KLAUNCH("k_hess_sweep", s, (k_hess_sweep<false><<<dim3(tiles_h, nsub), kHThreads, kHessSmem, s>>>(
                                     map_d, d_subs, norm, mask, fg, fg_idx, fg_count, d_status, WorkQueue{})));
    }
    return 0;
  }
  CUtensorMap map;
  if (encode_map(&map, norm, W, H, D, nsub, sweep_bw(rxy), sweep_bh(rxy)) != CUDA_SUCCESS) return -1;
  const unsigned tiles = ceil_div(W, kSX) * ceil_div(H, kSY);
  const size_t smem = sweep_smem_bytes(rxy);
  if (rz <= 5) {
    cudaFuncSetAttribute(k_dog_hess<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    KLAUNCH("k_dog_hess", s, (k_dog_hess<5><<<dim3(tiles, nsub), kSweepThreads, smem, s>>>(
                                 map, T, d_subs, norm, mask, fg, fg_idx, fg_count, d_status)));
  } else {
    cudaFuncSetAttribute(k_dog_hess<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    KLAUNCH("k_dog_hess", s, (k_dog_hess<8><<<dim3(tiles, nsub), kSweepThreads, smem, s>>>(
                                 map, T, d_subs, norm, mask, fg, fg_idx, fg_count, d_status)));
  }
  return 0;
}

}  // namespace hdog
