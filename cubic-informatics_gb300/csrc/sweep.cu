// sweep.cu -- fused DoG + Hessian + negative-definite test, one z-sweep per xy tile, sm_103a.
//
// Reference: src/3D/DoG3DFilter.cu (DoG3DFilter :431-437: x -> y -> z separable Gaussians
// with zero borders, `(small - large) * normalizer`) and src/3D/Hessian3DFilter_element.cu
// (HessianPositiveDefiniteWithElement :355-388: gradients of gradients with zero halos,
// Sylvester test).  The reference runs 16 full-volume passes here and keeps the DoG and
// six Hessian planes in memory; this kernel reads the normalized volume once and writes
// the uint8 mask plus a compact list of the foreground voxels' Hessian elements.
//
// A block owns a 64 x 16 output tile and sweeps z over the whole substack:
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

#include "kernels.cuh"

namespace hdog {

constexpr int kSX = 64, kSY = 16;                 // mask tile
constexpr int kEX = kSX + 4, kEY = kSY + 4;       // DoG tile with the Hessian halo
constexpr int kSweepThreads = 704;                // 22 warps
constexpr int kXQuads = kEX / 4;                  // 17 four-wide x-pass items per row
constexpr long long kWaitLimit = 1ll << 26;       // bounded mbarrier spin

__host__ __device__ inline int sweep_hx(int rxy) { return ((rxy + 2 + 3) / 4) * 4; }   // aligned x halo
__host__ __device__ inline int sweep_bw(int rxy) { return kSX + 2 * sweep_hx(rxy); }
__host__ __device__ inline int sweep_bh(int rxy) { return kSY + 4 + 2 * rxy; }

size_t sweep_smem_bytes(int rxy) {
  const size_t in = ((size_t)sweep_bw(rxy) * sweep_bh(rxy) * 4 + 127) / 128 * 128;
  const size_t xb = (size_t)sweep_bh(rxy) * kEX * sizeof(float2);
  const size_t ring = (size_t)5 * kEY * kEX * sizeof(float);
  return 2 * in + xb + ring + 64;
}

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

// One normalized slice (box bw x bh at (x, y, z, s)) into shared memory.
__device__ __forceinline__ void tma_slice(const CUtensorMap *map, float *dst, uint64_t *bar, int x, int y, int z, int s,
                                          uint32_t bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(s), "r"(smem_u32(bar))
      : "memory");
}

template <int RZ>
__global__ void __launch_bounds__(kSweepThreads, 1)
    k_dog_hess(const __grid_constant__ CUtensorMap map, const __grid_constant__ DogTaps T, const Sub *subs,
               const float *norm, uint8_t *mask, FgEntry *fg, unsigned long long *fg_count, int *status) {
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
      if (lane == 31 && tot) base = atomicAdd(&fg_count[blockIdx.y], (unsigned long long)tot);
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
        }
        base++;
      }
    }
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

// Whether the fused sweep handles these parameters (else the separate passes run).
bool sweep_supported(const DogTaps &T, int W, int max_smem) {
  const int rxy = max(T.r[0], T.r[2]), rz = max(T.r[1], T.r[3]);
  if (rxy > kMaxSweepRxy || rz > 8 || W % 4 != 0) return false;
  if ((int)sweep_smem_bytes(rxy) > max_smem) return false;
  return encode_fn() != nullptr;
}

int launch_dog_hess(const Sub *d_subs, int nsub, int W, int H, int D, const DogTaps &T, const float *norm,
                    uint8_t *mask, FgEntry *fg, unsigned long long *fg_count, int *d_status, cudaStream_t s) {
  const int rxy = max(T.r[0], T.r[2]), rz = max(T.r[1], T.r[3]);
  CUtensorMap map;
  const cuuint64_t dims[4] = {(cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D, (cuuint64_t)nsub};
  const cuuint64_t strides[3] = {(cuuint64_t)W * 4, (cuuint64_t)W * H * 4, (cuuint64_t)W * H * D * 4};
  const cuuint32_t box[4] = {(cuuint32_t)sweep_bw(rxy), (cuuint32_t)sweep_bh(rxy), 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float *>(norm), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return -1;
  const size_t smem = sweep_smem_bytes(rxy);
  const unsigned tiles = ceil_div(W, kSX) * ceil_div(H, kSY);
  cudaMemsetAsync(fg_count, 0, nsub * sizeof(unsigned long long), s);
  if (rz <= 5) {
    cudaFuncSetAttribute(k_dog_hess<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    KLAUNCH("k_dog_hess", s, (k_dog_hess<5><<<dim3(tiles, nsub), kSweepThreads, smem, s>>>(
                                 map, T, d_subs, norm, mask, fg, fg_count, d_status)));
  } else {
    cudaFuncSetAttribute(k_dog_hess<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    KLAUNCH("k_dog_hess", s, (k_dog_hess<8><<<dim3(tiles, nsub), kSweepThreads, smem, s>>>(
                                 map, T, d_subs, norm, mask, fg, fg_count, d_status)));
  }
  return 0;
}

}  // namespace hdog
