// norm.cu -- intensity normalization and the regional-erosion operator, sm_103a.
//
// Reference: src/3D/NormalizeFilter.cu (Normalize3DFilter :603-654) and
// src/3D/Erosion3DFilter.cu (Erosion3DFilter :260-268).
//
//   ero  = min over a (2rxy+1)^2 (2rz+1) box, dil = max over it    (nearest border)
//   ero_l = box mean of ero, dil_l = box mean of dil                 (nearest border)
//   norm = I >= min_intensity ? (I - ero_l) / (dil_l - ero_l) : 0
//
// Min and max are exact, so they are computed in whatever order is cheapest: the z pass
// first, straight from the raw slices, then x and y with a sparse-table (doubling)
// sliding window, O(log r) per voxel instead of O(r).  Erosion and dilation travel
// together as one packed u16 pair per voxel (low half min, high half max).
//
// The box means must round exactly like the reference, whose every pass is the
// sequential float sum `val = 0; for j in 0..2r: val += s[j]` times 1.0f/(2r+1):
//   x pass: the inputs are integers and every partial sum stays below 2^24 when
//           2r+1 <= 256, so the float chain is exact and equals an integer prefix-sum
//           difference; wider windows fall back to the literal chain;
//   y, z:   the literal chain, erosion and dilation side by side in one f32x2 add.
#include "kernels.cuh"

namespace hdog {

// ---------------------------------------------------------------- z pass (min/max)
// One thread per (x, y) column; slices at or past depth_valid read as zero (the zero
// tail HDoG3D_main.cpp:166-169 writes for a short last substack).  BORDER: 0 nearest
// (normalization), 1 zero (erosion operator).
template <int BORDER>
__global__ void k_minmax_z(const Sub *subs, int rz, uint32_t *mm) {
  const Sub S = subs[blockIdx.y];
  const int64_t plane = (int64_t)S.W * S.H;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= plane) return;
  const uint16_t *src = S.src + p;
  uint32_t *out = mm + S.vox + p;
  for (int z = 0; z < S.D; z++) {
    uint32_t lo = 0xFFFFu, hi = 0u;
    for (int j = -rz; j <= rz; j++) {
      int zz = z + j;
      uint32_t v;
      if (BORDER == 1 && (zz < 0 || zz >= S.D)) {
        v = 0;
      } else {
        zz = clampi(zz, 0, S.D - 1);
        v = zz < S.depth_valid ? (uint32_t)__ldg(src + zz * plane) : 0u;
      }
      lo = min(lo, v);
      hi = max(hi, v);
    }
    out[z * plane] = pack_mm(lo, hi);
  }
}

// Sparse-table sliding min/max over a window of L = 2r+1 entries of a smem line.
// buf0 holds n0 = count + 2r entries; after the call buf0 (or buf1) holds M_P, the
// combine of P = 2^floor(log2 L) consecutive entries.  Returns the buffer holding M_P.
__device__ __forceinline__ uint32_t *sparse_levels(uint32_t *buf0, uint32_t *buf1, int n0, int L,
                                                   int tid, int nthreads, int stride) {
  uint32_t *a = buf0, *b = buf1;
  int n = n0;
  for (int step = 1; 2 * step <= L; step *= 2) {
    const int m = n - step;
    for (int t = tid; t < m; t += nthreads) b[t * stride] = mm_combine(a[t * stride], a[(t + step) * stride]);
    __syncthreads();
    uint32_t *c = a; a = b; b = c;
    n = m;
  }
  return a;
}

// ---------------------------------------------------------------- x pass (min/max)
constexpr int kRowSeg = 256;   // outputs per block along x

template <int BORDER>
__global__ void k_minmax_x(const Sub *subs, int r, const uint32_t *in, uint32_t *out) {
  extern __shared__ uint32_t smx[];
  const Sub S = subs[blockIdx.y];
  const int segs = (S.W + kRowSeg - 1) / kRowSeg;
  const int64_t rows = (int64_t)S.H * S.D;
  const int64_t bid = blockIdx.x;
  if (bid >= rows * segs) return;
  const int64_t row = bid / segs;
  const int x0 = (int)(bid % segs) * kRowSeg;
  const int L = 2 * r + 1, n0 = kRowSeg + 2 * r;
  uint32_t *b0 = smx, *b1 = smx + n0;
  const uint32_t *line = in + S.vox + row * S.W;
  for (int t = threadIdx.x; t < n0; t += blockDim.x) {
    int x = x0 - r + t;
    uint32_t v;
    if (BORDER == 1 && (x < 0 || x >= S.W)) v = 0;
    else v = line[clampi(x, 0, S.W - 1)];
    b0[t] = v;
  }
  __syncthreads();
  int P = 1;
  while (2 * P <= L) P *= 2;
  uint32_t *m = sparse_levels(b0, b1, n0, L, threadIdx.x, blockDim.x, 1);
  const int t = threadIdx.x;
  const int x = x0 + t;
  if (x < S.W) out[S.vox + row * S.W + x] = mm_combine(m[t], m[t + L - P]);
}

// ---------------------------------------------------------------- y pass (min/max)
constexpr int kColTileX = 32;    // columns per block
constexpr int kColTileY = 64;    // output rows per block

template <int BORDER>
__global__ void k_minmax_y(const Sub *subs, int r, const uint32_t *in, uint32_t *out) {
  extern __shared__ uint32_t smy[];
  const Sub S = subs[blockIdx.y];
  const int tx_n = (S.W + kColTileX - 1) / kColTileX, ty_n = (S.H + kColTileY - 1) / kColTileY;
  const int64_t bid = blockIdx.x;
  if (bid >= (int64_t)tx_n * ty_n * S.D) return;
  const int z = (int)(bid / ((int64_t)tx_n * ty_n));
  const int rem = (int)(bid % ((int64_t)tx_n * ty_n));
  const int x0 = (rem % tx_n) * kColTileX, y0 = (rem / tx_n) * kColTileY;
  const int L = 2 * r + 1, n0 = kColTileY + 2 * r;
  uint32_t *b0 = smy, *b1 = smy + n0 * kColTileX;
  const int lx = threadIdx.x, ly = threadIdx.y;
  const int x = x0 + lx;
  const uint32_t *sl = in + S.vox + (int64_t)z * S.W * S.H;
  for (int t = ly; t < n0; t += blockDim.y) {
    int y = y0 - r + t;
    uint32_t v = 0;
    if (x < S.W) {
      if (BORDER == 1 && (y < 0 || y >= S.H)) v = 0;
      else v = sl[(int64_t)clampi(y, 0, S.H - 1) * S.W + x];
    }
    b0[t * kColTileX + lx] = v;
  }
  __syncthreads();
  // Doubling along y: each (lx, t) pair handled by thread (lx, t mod blockDim.y).
  uint32_t *a = b0, *b = b1;
  int n = n0, P = 1;
  for (int step = 1; 2 * step <= L; step *= 2) {
    const int m = n - step;
    for (int t = ly; t < m; t += blockDim.y)
      b[t * kColTileX + lx] = mm_combine(a[t * kColTileX + lx], a[(t + step) * kColTileX + lx]);
    __syncthreads();
    uint32_t *c = a; a = b; b = c;
    n = m;
    P = 2 * step;
  }
  if (x >= S.W) return;
  for (int t = ly; t < kColTileY; t += blockDim.y) {
    const int y = y0 + t;
    if (y < S.H) out[S.vox + ((int64_t)z * S.H + y) * S.W + x] =
        mm_combine(a[t * kColTileX + lx], a[(t + L - P) * kColTileX + lx]);
  }
}

// ---------------------------------------------------------------- x pass (box mean)
// Exact integer window sums (prefix-sum differences) when 2r+1 <= 256; the literal
// float chain otherwise.
__global__ void k_box_x(const Sub *subs, int r, const uint32_t *in, float2 *out) {
  extern __shared__ unsigned long long smb[];
  const Sub S = subs[blockIdx.y];
  const int segs = (S.W + kRowSeg - 1) / kRowSeg;
  const int64_t rows = (int64_t)S.H * S.D;
  const int64_t bid = blockIdx.x;
  if (bid >= rows * segs) return;
  const int64_t row = bid / segs;
  const int x0 = (int)(bid % segs) * kRowSeg;
  const int L = 2 * r + 1, n0 = kRowSeg + 2 * r;
  const float inv = 1.0f / (float)L;
  const uint32_t *line = in + S.vox + row * S.W;
  const int t = threadIdx.x;
  const int x = x0 + t;
  if (L <= 256) {
    // smb[0..n0]: exclusive prefix of packed (lo | hi << 32) sums; both halves stay
    // below 2^32 because n0 * 65535 < 2^32.
    __shared__ unsigned long long warp_tot[32];
    const int per = (n0 + blockDim.x - 1) / blockDim.x;
    const int beg = t * per, end = min(beg + per, n0);
    unsigned long long run = 0;
    for (int i = beg; i < end; i++) {
      uint32_t v = line[clampi(x0 - r + i, 0, S.W - 1)];
      smb[i] = run;
      run += (unsigned long long)(v & 0xFFFFu) | ((unsigned long long)(v >> 16) << 32);
    }
    // block exclusive scan of the per-thread totals
    unsigned long long inc = run;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if ((t & 31) >= o) inc += y;
    }
    if ((t & 31) == 31) warp_tot[t >> 5] = inc;
    __syncthreads();
    if (t < 32) {
      const int nw = blockDim.x >> 5;
      unsigned long long w = t < nw ? warp_tot[t] : 0ull, wi = w;
      for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
        if (t >= o) wi += y;
      }
      if (t < nw) warp_tot[t] = wi - w;
    }
    __syncthreads();
    const unsigned long long off = warp_tot[t >> 5] + (inc - run);
    for (int i = beg; i < end; i++) smb[i] += off;
    if (t == blockDim.x - 1) smb[n0] = off + run;
    __syncthreads();
    if (x < S.W) {
      const unsigned long long d = smb[t + L] - smb[t];
      const float lo = (float)(uint32_t)(d & 0xFFFFFFFFull), hi = (float)(uint32_t)(d >> 32);
      out[S.vox + row * S.W + x] = make_float2(lo * inv, hi * inv);
    }
  } else {
    float2 *sf = reinterpret_cast<float2 *>(smb);
    for (int i = t; i < n0; i += blockDim.x) {
      uint32_t v = line[clampi(x0 - r + i, 0, S.W - 1)];
      sf[i] = make_float2((float)(v & 0xFFFFu), (float)(v >> 16));
    }
    __syncthreads();
    if (x < S.W) {
      float2 acc = make_float2(0.f, 0.f);
      for (int j = 0; j < L; j++) acc = add2(acc, sf[t + j]);
      out[S.vox + row * S.W + x] = mul2(acc, make_float2(inv, inv));
    }
  }
}

// ---------------------------------------------------------------- y / z passes (box mean)
// Register-blocked sequential sums: a thread produces K consecutive outputs along the
// axis; slot (u + k) % K of a K-entry rotating window feeds output k at tap u of each
// block of K taps, so the window never moves between registers.  Every output still
// sums its 2r+1 inputs from 0.0f in the reference order.
constexpr int kBoxK = 8;

template <class LoadF>
__device__ __forceinline__ void box_chain(int c0, int r, LoadF load, float2 (&acc)[kBoxK]) {
  float2 win[kBoxK];
#pragma unroll
  for (int k = 0; k < kBoxK; k++) { win[k] = load(c0 - r + k); acc[k] = make_float2(0.f, 0.f); }
  const int L = 2 * r + 1;
  for (int jb = 0; jb < L; jb += kBoxK) {
#pragma unroll
    for (int u = 0; u < kBoxK; u++) {
      const int j = jb + u;
      if (j < L) {
#pragma unroll
        for (int k = 0; k < kBoxK; k++) acc[k] = add2(acc[k], win[(u + k) % kBoxK]);
        win[u] = load(c0 - r + j + kBoxK);
      }
    }
  }
}

__global__ void k_box_y(const Sub *subs, int r, const float2 *in, float2 *out) {
  const Sub S = subs[blockIdx.y];
  const int rows_per_blk = blockDim.y * kBoxK;
  const int tx_n = (S.W + 31) / 32, ty_n = (S.H + rows_per_blk - 1) / rows_per_blk;
  const int64_t bid = blockIdx.x;
  if (bid >= (int64_t)tx_n * ty_n * S.D) return;
  const int z = (int)(bid / ((int64_t)tx_n * ty_n));
  const int rem = (int)(bid % ((int64_t)tx_n * ty_n));
  const int x = (rem % tx_n) * 32 + threadIdx.x;
  const int y0 = (rem / tx_n) * rows_per_blk + threadIdx.y * kBoxK;
  if (x >= S.W || y0 >= S.H) return;
  const float2 *col = in + S.vox + (int64_t)z * S.W * S.H + x;
  const int H = S.H, W = S.W;
  float2 acc[kBoxK];
  box_chain(y0, r, [&](int y) { return col[(int64_t)clampi(y, 0, H - 1) * W]; }, acc);
  const float inv = 1.0f / (float)(2 * r + 1);
  float2 *o = out + S.vox + (int64_t)z * S.W * S.H + x;
#pragma unroll
  for (int k = 0; k < kBoxK; k++)
    if (y0 + k < H) o[(int64_t)(y0 + k) * W] = mul2(acc[k], make_float2(inv, inv));
}

// z pass of the box mean fused with Normalize3DKernel (NormalizeFilter.cu:571-586).
__global__ void k_box_z_norm(const Sub *subs, int rz, float min_intensity, const float2 *in,
                             float *norm) {
  const Sub S = subs[blockIdx.y];
  const int64_t plane = (int64_t)S.W * S.H;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= plane) return;
  const float2 *col = in + S.vox + p;
  const int D = S.D;
  const float inv = 1.0f / (float)(2 * rz + 1);
  for (int z0 = 0; z0 < D; z0 += kBoxK) {
    float2 acc[kBoxK];
    box_chain(z0, rz, [&](int z) { return col[clampi(z, 0, D - 1) * plane]; }, acc);
#pragma unroll
    for (int k = 0; k < kBoxK; k++) {
      const int z = z0 + k;
      if (z < D) {
        const float2 el = mul2(acc[k], make_float2(inv, inv));
        const float v = z < S.depth_valid ? (float)__ldg(S.src + z * plane + p) : 0.0f;
        norm[S.vox + z * plane + p] = (v >= min_intensity) ? (v - el.x) / (el.y - el.x) : 0.0f;
      }
    }
  }
}

// Copy3DKernel (NormalizeFilter.cu:588-601), used when a normalization radius is 0.
__global__ void k_copy_norm(const Sub *subs, float min_intensity, float *norm) {
  const Sub S = subs[blockIdx.y];
  const int64_t n = (int64_t)S.W * S.H * S.D, plane = (int64_t)S.W * S.H;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int z = (int)(i / plane);
  const float v = z < S.depth_valid ? (float)S.src[i] : 0.0f;
  norm[S.vox + i] = (v >= min_intensity) ? v : 0.0f;
}

__global__ void k_unpack_lo(const Sub *subs, const uint32_t *mm, uint16_t *dst) {
  const Sub S = subs[blockIdx.y];
  const int64_t n = (int64_t)S.W * S.H * S.D;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dst[S.vox + i] = (uint16_t)(mm[S.vox + i] & 0xFFFFu);
}

// ---------------------------------------------------------------- launchers
static size_t minmax_y_smem(int r) { return (size_t)2 * (kColTileY + 2 * r) * kColTileX * sizeof(uint32_t); }

void launch_minmax_z(const Sub *d_subs, int nsub, int max_plane, int rz, uint32_t *mm, cudaStream_t s) {
  dim3 grid(ceil_div(max_plane, 256), nsub);
  KLAUNCH("k_minmax_z", s, (k_minmax_z<0><<<grid, 256, 0, s>>>(d_subs, rz, mm)));
}

void launch_minmax_x(const Sub *d_subs, int nsub, int64_t max_rows, int max_w, int r,
                     const uint32_t *in, uint32_t *out, cudaStream_t s) {
  dim3 grid((unsigned)(max_rows * ceil_div(max_w, kRowSeg)), nsub);
  size_t smem = (size_t)2 * (kRowSeg + 2 * r) * sizeof(uint32_t);
  KLAUNCH("k_minmax_x", s, (k_minmax_x<0><<<grid, kRowSeg, smem, s>>>(d_subs, r, in, out)));
}

void launch_minmax_y(const Sub *d_subs, int nsub, int max_w, int max_h, int max_d, int r,
                     const uint32_t *in, uint32_t *out, cudaStream_t s) {
  dim3 grid((unsigned)((int64_t)ceil_div(max_w, kColTileX) * ceil_div(max_h, kColTileY) * max_d), nsub);
  size_t smem = minmax_y_smem(r);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k_minmax_y<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  KLAUNCH("k_minmax_y", s, (k_minmax_y<0><<<grid, dim3(kColTileX, 8), smem, s>>>(d_subs, r, in, out)));
}

void launch_box_x(const Sub *d_subs, int nsub, int64_t max_rows, int max_w, int r,
                  const uint32_t *in, float2 *out, cudaStream_t s) {
  dim3 grid((unsigned)(max_rows * ceil_div(max_w, kRowSeg)), nsub);
  size_t smem = (size_t)(kRowSeg + 2 * r + 1) * sizeof(unsigned long long);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k_box_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  KLAUNCH("k_box_x", s, (k_box_x<<<grid, kRowSeg, smem, s>>>(d_subs, r, in, out)));
}

void launch_box_y(const Sub *d_subs, int nsub, int max_w, int max_h, int max_d, int r,
                  const float2 *in, float2 *out, cudaStream_t s) {
  const int by = 4;
  dim3 grid((unsigned)((int64_t)ceil_div(max_w, 32) * ceil_div(max_h, by * kBoxK) * max_d), nsub);
  KLAUNCH("k_box_y", s, (k_box_y<<<grid, dim3(32, by), 0, s>>>(d_subs, r, in, out)));
}

void launch_box_z_norm(const Sub *d_subs, int nsub, int max_plane, int rz, float min_intensity,
                       const float2 *in, float *norm, cudaStream_t s) {
  dim3 grid(ceil_div(max_plane, 128), nsub);
  KLAUNCH("k_box_z_norm", s, (k_box_z_norm<<<grid, 128, 0, s>>>(d_subs, rz, min_intensity, in, norm)));
}

void launch_copy_norm(const Sub *d_subs, int nsub, int64_t max_n, float min_intensity, float *norm,
                      cudaStream_t s) {
  dim3 grid(ceil_div(max_n, 256), nsub);
  KLAUNCH("k_copy_norm", s, (k_copy_norm<<<grid, 256, 0, s>>>(d_subs, min_intensity, norm)));
}

// Erosion3DFilter: min with a zero border.  Min is separable and exact, so z -> x -> y
// gives the reference's x -> y -> z result.  `tmp` holds two packed u32 volumes.
void launch_erosion(const Sub *d_subs, int nsub, int max_w, int max_h, int max_d, int64_t max_rows,
                    int rxy, int rz, const uint16_t *src_override, uint16_t *tmp_u16, uint16_t *dst,
                    cudaStream_t s) {
  (void)src_override;
  uint32_t *a = reinterpret_cast<uint32_t *>(tmp_u16);
  const int64_t max_n = max_rows * max_w;
  uint32_t *b = a + max_n * nsub;
  const int max_plane = max_w * max_h;
  KLAUNCH("k_minmax_z", s, (k_minmax_z<1><<<dim3(ceil_div(max_plane, 256), nsub), 256, 0, s>>>(d_subs, rz, a)));
  size_t smx = (size_t)2 * (kRowSeg + 2 * rxy) * sizeof(uint32_t);
  KLAUNCH("k_minmax_x", s, (k_minmax_x<1><<<dim3((unsigned)(max_rows * ceil_div(max_w, kRowSeg)), nsub), kRowSeg, smx, s>>>(d_subs, rxy, a, b)));
  size_t smy = minmax_y_smem(rxy);
  if (smy > 48 * 1024) cudaFuncSetAttribute(k_minmax_y<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smy);
  KLAUNCH("k_minmax_y", s, (k_minmax_y<1><<<dim3((unsigned)((int64_t)ceil_div(max_w, kColTileX) * ceil_div(max_h, kColTileY) * max_d), nsub),
                  dim3(kColTileX, 8), smy, s>>>(d_subs, rxy, b, a)));
  KLAUNCH("k_unpack_lo", s, (k_unpack_lo<<<dim3(ceil_div(max_n, 256), nsub), 256, 0, s>>>(d_subs, a, dst)));
}

}  // namespace hdog
