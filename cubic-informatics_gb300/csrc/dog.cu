// dog.cu -- difference of Gaussians and the Hessian negative-definite mask, sm_103a.
//
// Reference: src/3D/DoG3DFilter.cu (DoG3DFilter :431-437) and
// src/3D/Hessian3DFilter_element.cu (HessianPositiveDefiniteWithElement :355-388).
//
// DoG: both Gaussian scales run together, the small one in the .x lane and the large one
// in the .y lane of an f32x2, so one packed FMA advances both chains.  Each output is the
// reference's chain `sum = 0; for j = -r..r: sum = fma(k[r-j], s[x+j], sum)` with a zero
// border, x then y then z; taps that exist for one scale only run as scalar FMAs on its
// lane, so neither chain sees an extra term.
//
// Hessian: gradients of gradients with a zero halo at every step, computed from a dog
// tile staged in shared memory; only the uint8 mask is written (the six elements are
// written only on request, for stage-wise checks).
#include "kernels.cuh"

namespace hdog {

constexpr int kConvSeg = 256;   // x outputs per block
constexpr int kConvK = 8;       // outputs per thread along y / z

// ---------------------------------------------------------------- x pass
__global__ void k_conv_x(const Sub *subs, const __grid_constant__ DogTaps T, const float *in, float2 *out) {
  extern __shared__ float scx[];
  const Sub S = subs[blockIdx.y];
  const int segs = (S.W + kConvSeg - 1) / kConvSeg;
  const int64_t rows = (int64_t)S.H * S.D;
  const int64_t bid = blockIdx.x;
  if (bid >= rows * segs) return;
  const int64_t row = bid / segs;
  const int x0 = (int)(bid % segs) * kConvSeg;
  const int ra = T.r[0], rb = T.r[2], rm = max(ra, rb);
  const int n0 = kConvSeg + 2 * rm;
  const float *line = in + S.vox + row * S.W;
  for (int t = threadIdx.x; t < n0; t += blockDim.x) {
    const int x = x0 - rm + t;
    scx[t] = (x >= 0 && x < S.W) ? line[x] : 0.0f;
  }
  __syncthreads();
  const int t = threadIdx.x, x = x0 + t;
  if (x >= S.W) return;
  float2 acc = make_float2(0.f, 0.f);
  const float *s = scx + t + rm;
  for (int j = -rm; j <= rm; j++) {
    const bool aa = j >= -ra && j <= ra, ab = j >= -rb && j <= rb;
    const float v = s[j];
    if (aa && ab) acc = fma2(make_float2(T.k[0][ra - j], T.k[2][rb - j]), make_float2(v, v), acc);
    else if (ab) acc.y = __fmaf_rn(T.k[2][rb - j], v, acc.y);
    else if (aa) acc.x = __fmaf_rn(T.k[0][ra - j], v, acc.x);
  }
  out[S.vox + row * S.W + x] = acc;
}

// Register-blocked FMA chains along y or z for both scales (lane x: taps ka/radius ra,
// lane y: taps kb/radius rb).  Same rotating-window scheme as the box sums.
template <class LoadF>
__device__ __forceinline__ void conv_chain(int c0, const float *ka, int ra, const float *kb, int rb,
                                           LoadF load, float2 (&acc)[kConvK]) {
  const int rm = max(ra, rb), L = 2 * rm + 1;
  float2 win[kConvK];
#pragma unroll
  for (int k = 0; k < kConvK; k++) { win[k] = load(c0 - rm + k); acc[k] = make_float2(0.f, 0.f); }
  for (int jb = 0; jb < L; jb += kConvK) {
#pragma unroll
    for (int u = 0; u < kConvK; u++) {
      const int j = jb + u;
      if (j < L) {
        const int jj = j - rm;
        const bool aa = jj >= -ra && jj <= ra, ab = jj >= -rb && jj <= rb;
        if (aa && ab) {
          const float2 kk = make_float2(ka[ra - jj], kb[rb - jj]);
#pragma unroll
          for (int k = 0; k < kConvK; k++) acc[k] = fma2(kk, win[(u + k) % kConvK], acc[k]);
        } else if (ab) {
          const float kk = kb[rb - jj];
#pragma unroll
          for (int k = 0; k < kConvK; k++) acc[k].y = __fmaf_rn(kk, win[(u + k) % kConvK].y, acc[k].y);
        } else if (aa) {
          const float kk = ka[ra - jj];
#pragma unroll
          for (int k = 0; k < kConvK; k++) acc[k].x = __fmaf_rn(kk, win[(u + k) % kConvK].x, acc[k].x);
        }
        win[u] = load(c0 - rm + j + kConvK);
      }
    }
  }
}

// ---------------------------------------------------------------- y pass
__global__ void k_conv_y(const Sub *subs, const __grid_constant__ DogTaps T, const float2 *in, float2 *out) {
  const Sub S = subs[blockIdx.y];
  const int rows_per_blk = blockDim.y * kConvK;
  const int tx_n = (S.W + 31) / 32, ty_n = (S.H + rows_per_blk - 1) / rows_per_blk;
  const int64_t bid = blockIdx.x;
  if (bid >= (int64_t)tx_n * ty_n * S.D) return;
  const int z = (int)(bid / ((int64_t)tx_n * ty_n));
  const int rem = (int)(bid % ((int64_t)tx_n * ty_n));
  const int x = (rem % tx_n) * 32 + threadIdx.x;
  const int y0 = (rem / tx_n) * rows_per_blk + threadIdx.y * kConvK;
  if (x >= S.W || y0 >= S.H) return;
  const int W = S.W, H = S.H;
  const float2 *col = in + S.vox + (int64_t)z * W * H + x;
  float2 acc[kConvK];
  conv_chain(y0, T.k[0], T.r[0], T.k[2], T.r[2],
             [&](int y) { return (y >= 0 && y < H) ? col[(int64_t)y * W] : make_float2(0.f, 0.f); }, acc);
  float2 *o = out + S.vox + (int64_t)z * W * H + x;
#pragma unroll
  for (int k = 0; k < kConvK; k++)
    if (y0 + k < H) o[(int64_t)(y0 + k) * W] = acc[k];
}

// ---------------------------------------------------------------- z pass + subtract
// NormalizeSubtract3DKernel (DoG3DFilter.cu:346-354): dog = (small - large) * normalizer.
__global__ void k_conv_z_dog(const Sub *subs, const __grid_constant__ DogTaps T, const float2 *in, float *dog) {
  const Sub S = subs[blockIdx.y];
  const int64_t plane = (int64_t)S.W * S.H;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= plane) return;
  const int D = S.D;
  const float2 *col = in + S.vox + p;
  for (int z0 = 0; z0 < D; z0 += kConvK) {
    float2 acc[kConvK];
    conv_chain(z0, T.k[1], T.r[1], T.k[3], T.r[3],
               [&](int z) { return (z >= 0 && z < D) ? col[z * plane] : make_float2(0.f, 0.f); }, acc);
#pragma unroll
    for (int k = 0; k < kConvK; k++) {
      const int z = z0 + k;
      if (z < D) dog[S.vox + z * plane + p] = __fmul_rn(__fsub_rn(acc[k].x, acc[k].y), T.normalizer);
    }
  }
}

// ---------------------------------------------------------------- Hessian + PD mask
constexpr int kHX = 32, kHY = 8, kHZ = 8;          // outputs per block
constexpr int kDX = kHX + 4, kDY = kHY + 4, kDZ = kHZ + 4;   // dog tile (halo 2)
constexpr int kGX = kHX + 2, kGY = kHY + 2, kGZ = kHZ + 2;   // gradient tiles (halo 1)

__global__ void __launch_bounds__(256) k_hessian_pd(const Sub *subs, const float *dog, uint8_t *mask,
                                                    float *hess6) {
  extern __shared__ float sh[];
  float *sd = sh;                               // kDZ*kDY*kDX
  float *sgx = sd + kDZ * kDY * kDX;            // kGZ*kGY*kGX each
  float *sgy = sgx + kGZ * kGY * kGX;
  float *sgz = sgy + kGZ * kGY * kGX;
  const Sub S = subs[blockIdx.y];
  const int nx = (S.W + kHX - 1) / kHX, ny = (S.H + kHY - 1) / kHY, nz = (S.D + kHZ - 1) / kHZ;
  const int64_t bid = blockIdx.x;
  if (bid >= (int64_t)nx * ny * nz) return;
  const int bx = (int)(bid % nx), by = (int)((bid / nx) % ny), bz = (int)(bid / ((int64_t)nx * ny));
  const int x0 = bx * kHX, y0 = by * kHY, z0 = bz * kHZ;
  const int W = S.W, H = S.H, D = S.D;
  const int64_t plane = (int64_t)W * H;
  const float *f = dog + S.vox;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nt = blockDim.x * blockDim.y;
  for (int i = tid; i < kDZ * kDY * kDX; i += nt) {
    const int lx = i % kDX, ly = (i / kDX) % kDY, lz = i / (kDX * kDY);
    const int x = x0 - 2 + lx, y = y0 - 2 + ly, z = z0 - 2 + lz;
    sd[i] = (x >= 0 && x < W && y >= 0 && y < H && z >= 0 && z < D) ? f[z * plane + (int64_t)y * W + x] : 0.0f;
  }
  __syncthreads();
  for (int i = tid; i < kGZ * kGY * kGX; i += nt) {
    const int lx = i % kGX, ly = (i / kGX) % kGY, lz = i / (kGX * kGY);
    const int x = x0 - 1 + lx, y = y0 - 1 + ly, z = z0 - 1 + lz;
    const bool in = x >= 0 && x < W && y >= 0 && y < H && z >= 0 && z < D;
    const int c = ((lz + 1) * kDY + (ly + 1)) * kDX + (lx + 1);
    sgx[i] = in ? cdiff(sd[c + 1], sd[c - 1]) : 0.0f;
    sgy[i] = in ? cdiff(sd[c + kDX], sd[c - kDX]) : 0.0f;
    sgz[i] = in ? cdiff(sd[c + kDX * kDY], sd[c - kDX * kDY]) : 0.0f;
  }
  __syncthreads();
  const int lx = threadIdx.x, ly = threadIdx.y;
  const int x = x0 + lx, y = y0 + ly;
  if (x >= W || y >= H) return;
  const int64_t n = S.vox;  // plane offset base for optional planes
  const int64_t nvox = (int64_t)W * H * D;
  for (int lz = 0; lz < kHZ; lz++) {
    const int z = z0 + lz;
    if (z >= D) break;
    const int g = ((lz + 1) * kGY + (ly + 1)) * kGX + (lx + 1);
    const int sy = kGX, sz = kGX * kGY;
    const float hxx = cdiff(sgx[g + 1], sgx[g - 1]);
    const float hxy = cdiff(sgx[g + sy], sgx[g - sy]);
    const float hxz = cdiff(sgx[g + sz], sgx[g - sz]);
    const float hyy = cdiff(sgy[g + sy], sgy[g - sy]);
    const float hyz = cdiff(sgy[g + sz], sgy[g - sz]);
    const float hzz = cdiff(sgz[g + sz], sgz[g - sz]);
    const int64_t i = z * plane + (int64_t)y * W + x;
    mask[n + i] = pd_test(hxx, hxy, hxz, hyy, hyz, hzz) ? 1 : 0;
    if (hess6) {
      float *hp = hess6 + 6 * S.vox + i;
      hp[0] = hxx; hp[nvox] = hxy; hp[2 * nvox] = hxz;
      hp[3 * nvox] = hyy; hp[4 * nvox] = hyz; hp[5 * nvox] = hzz;
    }
  }
}

// ---------------------------------------------------------------- launchers
void launch_dog(const Sub *d_subs, int nsub, int max_w, int max_h, int max_d, int64_t max_rows,
                const DogTaps &T, const float *norm, float2 *t0, float2 *t1, float *dog, cudaStream_t s) {
  const int rm = max(T.r[0], T.r[2]);
  size_t smx = (size_t)(kConvSeg + 2 * rm) * sizeof(float);
  KLAUNCH("k_conv_x", s, (k_conv_x<<<dim3((unsigned)(max_rows * ceil_div(max_w, kConvSeg)), nsub), kConvSeg, smx, s>>>(d_subs, T, norm, t0)));
  const int by = 4;
  KLAUNCH("k_conv_y", s, (k_conv_y<<<dim3((unsigned)((int64_t)ceil_div(max_w, 32) * ceil_div(max_h, by * kConvK) * max_d), nsub),
             dim3(32, by), 0, s>>>(d_subs, T, t0, t1)));
  KLAUNCH("k_conv_z_dog", s, (k_conv_z_dog<<<dim3(ceil_div((int64_t)max_w * max_h, 128), nsub), 128, 0, s>>>(d_subs, T, t1, dog)));
}

void launch_hessian_pd(const Sub *d_subs, int nsub, int max_w, int max_h, int max_d, const float *dog,
                       uint8_t *mask, float *hess6, cudaStream_t s) {
  const size_t smem = (size_t)(kDZ * kDY * kDX + 3 * kGZ * kGY * kGX) * sizeof(float);
  cudaFuncSetAttribute(k_hessian_pd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int64_t tiles = (int64_t)ceil_div(max_w, kHX) * ceil_div(max_h, kHY) * ceil_div(max_d, kHZ);
  KLAUNCH("k_hessian_pd", s, (k_hessian_pd<<<dim3((unsigned)tiles, nsub), dim3(kHX, kHY), smem, s>>>(d_subs, dog, mask, hess6)));
}

}  // namespace hdog
