// soft.cu -- the differentiable HDoG chain, sm_103a: forward and hand-written adjoint of
// normalize -> DoG -> Hessian -> relaxed positive-definiteness score at sample points.
//
// Forward stages follow the reference's (NormalizeFilter.cu:537-654, DoG3DFilter.cu:70-437,
// Hessian3DFilter_element.cu:22-388) with its borders, in float32 without the bit-exact
// summation orders of the detection path: min / max and box means with nearest borders,
// separable Gaussians with zero borders (one sigma per axis and scale), central
// differences of central differences with zeros outside the volume, and the mask test
// xx < 0, xx yy - xy^2 > 0, det < 0 relaxed to a product of sigmoids of the minors scaled
// by tau, tau^2, tau^3.  Loss = mean score at the positive points - mean score at the
// negative points.
//
// Backward recomputes every intermediate from the input, or (the _kept entry) takes the
// forward chain's intermediates from the workspace the forward call filled, which the
// backward does not overwrite, and runs the adjoints in reverse: the score's derivative scattered through the
// Hessian stencil into a DoG-shaped gradient; for the sigmas, the derivative-of-Gaussian
// taps (d t_k / d sigma = t_k (k^2 - sum_j t_j j^2) / sigma^3 for the normalized taps) on
// one axis and the plain taps on the others, dotted with that gradient, plus the
// normalizer's term; for the input, the transposed separable Gaussians (the taps are
// symmetric and the borders zero, so the transpose is the same correlation), the
// normalization's quotient rule, the transposed box means (a gather that counts how often
// the nearest border repeats each edge value) and the transposed min / max filters (each
// window's gradient goes to its first extreme, recomputed from the filter's input).
// Tap radii are (int)(2 sigma + 0.5), held fixed for the derivatives.
//
// The windowed passes (and their transposes) run from shared-memory tiles that stage a line
// segment or column slab with the window's reach once (k_soft_pass_x / _yz, k_soft_adj_x /
// _yz, k_soft_ext_yz, k_soft_ext_adj_yz), and fall back to the untiled kernels for reaches
// above kSoftTileMaxR.  Box means and Gaussians fold each output's window in one fixed order:
// the float32 sigma gradients are sensitive to the last bits of the normalized volume, so
// that order is kept.  Min / max windows and their first extremes, which do not round, come
// from doubling in the tile.
#include <cmath>

#include "kernels.cuh"

namespace hdog {

constexpr int kSoftMaxRadius = 31;
constexpr int kSoftMaxTaps = 2 * kSoftMaxRadius + 1;
struct SoftTaps {
  float k[kSoftMaxTaps];
  int r;
};
enum { kMin = 0, kMax = 1, kBox = 2, kConv = 3 };
struct SoftGeom {
  int W, H, D;
};

__device__ __forceinline__ void soft_axis(const SoftGeom &g, int axis, int64_t i, int &c, int64_t &stride, int &n) {
  const int x = (int)(i % g.W), y = (int)((i / g.W) % g.H), z = (int)(i / ((int64_t)g.W * g.H));
  if (axis == 0) { c = x; stride = 1; n = g.W; }
  else if (axis == 1) { c = y; stride = g.W; n = g.H; }
  else { c = z; stride = (int64_t)g.W * g.H; n = g.D; }
}

// One separable pass along `axis` (0 x, 1 y, 2 z): min / max / box mean with nearest
// borders, or the correlation with T (zero border).
__global__ void k_soft_pass(const float *in, float *out, SoftGeom g, int axis, int mode, int r, SoftTaps T, int64_t N) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int c, n;
  int64_t s;
  soft_axis(g, axis, i, c, s, n);
  const float *line = in + (i - (int64_t)c * s);
  float acc;
  if (mode == kConv) {
    acc = 0.0f;
    for (int j = -T.r; j <= T.r; j++) {
      const int p = c + j;
      if (p >= 0 && p < n) acc = __fmaf_rn(T.k[j + T.r], line[(int64_t)p * s], acc);
    }
  } else if (mode == kBox) {
    acc = 0.0f;
    for (int j = -r; j <= r; j++) acc += line[(int64_t)clampi(c + j, 0, n - 1) * s];
    acc = acc / (float)(2 * r + 1);
  } else {
    acc = line[(int64_t)clampi(c - r, 0, n - 1) * s];
    for (int j = -r + 1; j <= r; j++) {
      const float v = line[(int64_t)clampi(c + j, 0, n - 1) * s];
      acc = mode == kMin ? fminf(acc, v) : fmaxf(acc, v);
    }
  }
  out[i] = acc;
}

// The same pass from a shared-memory tile: a block stages the inputs of its outputs once
// (along x a row segment of kSoftTileX outputs plus the window's reach on each side; along y
// or z a 32-column slab of kSoftTileYZ outputs plus the reach), out-of-line positions already
// clamped (min / max / box) or zero (conv), and every output folds its window in the same
// order and with the same operations as k_soft_pass, so the results are identical; only
// the repeated global loads of overlapping windows are gone.  For reaches up to
// kSoftTileMaxR.
constexpr int kSoftTileX = 256, kSoftTileYZ = 64, kSoftTileMaxR = 64;

__device__ __forceinline__ float soft_fold(const float *w, int step, int c, int n, int mode, int R, const SoftTaps &T) {
  // w[k * step] is the input at line position c - R + k
  float acc;
  if (mode == kConv) {
    acc = 0.0f;
    for (int j = -R; j <= R; j++) {
      const int p = c + j;
      if (p >= 0 && p < n) acc = __fmaf_rn(T.k[j + R], w[(j + R) * step], acc);
    }
  } else if (mode == kBox) {
    acc = 0.0f;
    for (int j = -R; j <= R; j++) acc += w[(j + R) * step];
    acc = acc / (float)(2 * R + 1);
  } else {
    acc = w[0];
    for (int j = -R + 1; j <= R; j++) {
      const float v = w[(j + R) * step];
      acc = mode == kMin ? fminf(acc, v) : fmaxf(acc, v);
    }
  }
  return acc;
}

__device__ __forceinline__ float soft_stage(const float *line, int64_t s, int p, int n, int mode) {
  if (mode == kConv) return (p >= 0 && p < n) ? line[(int64_t)p * s] : 0.0f;
  return line[(int64_t)clampi(p, 0, n - 1) * s];
}

// Min / max windows from the staged tile by doubling: after the steps with spans 1, 2, ..., q
// an entry holds the extreme of the q staged values from it on, where q is the largest power
// of two <= w = 2R + 1; a window [t, t + 2R] is then the extreme of the entries t and
// t + w - q (two spans that overlap and cover it).  Min and max do not round, so the values
// equal the sequential fold's (for inputs without NaN).  With indices, an entry also carries
// the staged position of its span's first extreme: a later span replaces it only when
// strictly better, which keeps the first extreme of the union (a tie inside the overlap is
// already the earlier span's).  Along y and z a block of 32 x 16 threads doubles a slab of
// kSoftTileYZ + 2R rows (R <= kSoftExtMaxR), kSoftExtPer rows per thread.
constexpr int kSoftExtMaxR = 32, kSoftExtPer = (kSoftTileYZ + 2 * kSoftExtMaxR) / 16;

__device__ __forceinline__ float soft_ext(float a, float b, bool is_max) { return is_max ? fmaxf(a, b) : fminf(a, b); }

__device__ __forceinline__ void soft_ext_at(float &a, int &ia, float b, int ib, bool is_max) {
  if (is_max ? b > a : b < a) {
    a = b;
    ia = ib;
  }
}

__device__ __forceinline__ int soft_span(int R) {   // the largest power of two <= 2R + 1
  return 1 << (31 - __clz(2 * R + 1));
}

// Dot products as compensated float32 sums (GB300's FP64 pipe is a small fraction of its
// FP32 rate): a product a b is split exactly into p + e (p = a b rounded, e = fma(a, b, -p)),
// added to a running hi + lo by Knuth's TwoSum (the rounding error of hi + p goes to lo), and
// per warp the pairs combine the same way before one conversion to double; the relative error
// of a thread's or warp's sum is about 2^-48, against 2^-53 per addition of a double sum.
__device__ __forceinline__ void soft_two_sum(float &hi, float &lo, float v) {
  const float s = __fadd_rn(hi, v), bb = __fsub_rn(s, hi);
  lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(v, bb)));
  hi = s;
}

__device__ __forceinline__ void soft_dot_add(float &hi, float &lo, float a, float b) {
  const float p = __fmul_rn(a, b);
  lo = __fadd_rn(lo, __fmaf_rn(a, b, -p));
  soft_two_sum(hi, lo, p);
}

// the warp's (hi, lo) pairs summed into lane 0's, returned as a double there
__device__ __forceinline__ double soft_warp_dot(float hi, float lo) {
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_down_sync(0xFFFFFFFFu, hi, o), l2 = __shfl_down_sync(0xFFFFFFFFu, lo, o);
    lo = __fadd_rn(lo, l2);
    soft_two_sum(hi, lo, h2);
  }
  return (double)hi + (double)lo;
}

// along x: a block takes the same segment of kSoftRowsX consecutive rows (so each thread has
// several loads in flight before the barrier), one output per thread and row
constexpr int kSoftRowsX = 4;

__global__ void __launch_bounds__(kSoftTileX) k_soft_pass_x(const float *in, float *out, SoftGeom g, int mode, int R,
                                                            SoftTaps T) {
  __shared__ float tile[kSoftRowsX][kSoftTileX + 2 * kSoftTileMaxR];
  const int nseg = (g.W + kSoftTileX - 1) / kSoftTileX;
  const int64_t row0 = (int64_t)(blockIdx.x / nseg) * kSoftRowsX;
  const int nr = (int)min((int64_t)kSoftRowsX, (int64_t)g.H * g.D - row0);
  const int x0 = (int)(blockIdx.x % nseg) * kSoftTileX, t = threadIdx.x;
  const int L = kSoftTileX + 2 * R;
  for (int r = 0; r < nr; r++)
    for (int k = t; k < L; k += kSoftTileX) tile[r][k] = soft_stage(in + (row0 + r) * g.W, 1, x0 - R + k, g.W, mode);
  __syncthreads();
  const int x = x0 + t;
  if (mode == kMin || mode == kMax) {
    const bool is_max = mode == kMax;
    const int q_end = soft_span(R);
    for (int q = 1; q < q_end; q *= 2) {
      const int lim = L - 2 * q + 1;   // entries whose span of 2q stays inside the tile
      float a[kSoftRowsX][2];
#pragma unroll
      for (int r = 0; r < kSoftRowsX; r++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int k = t + h * kSoftTileX;
          a[r][h] = r < nr && k < lim ? soft_ext(tile[r][k], tile[r][k + q], is_max) : 0.0f;
        }
      __syncthreads();
#pragma unroll
      for (int r = 0; r < kSoftRowsX; r++)
#pragma unroll
        for (int h = 0; h < 2; h++)
          if (r < nr && t + h * kSoftTileX < lim) tile[r][t + h * kSoftTileX] = a[r][h];
      __syncthreads();
    }
    if (x < g.W)
      for (int r = 0; r < nr; r++)
        out[(row0 + r) * g.W + x] = soft_ext(tile[r][t], tile[r][t + 2 * R + 1 - q_end], is_max);
    return;
  }
  if (x < g.W)
    for (int r = 0; r < nr; r++) out[(row0 + r) * g.W + x] = soft_fold(tile[r] + t, 1, x, g.W, mode, R, T);
}

// along y (AXIS 1) or z (AXIS 2): a block of 32 x 8 threads owns 32 columns and
// kSoftTileYZ outputs of each; thread (tx, ty) computes outputs ty, ty + 8, ...  The epilogue
// stores the outputs (kEpiStore); or stores scale * (aux - output), the DoG difference
// (kEpiDiff); or stores nothing and adds sum(output * aux) over the block's outputs to
// *dot_out (kEpiDot; a double, from compensated float32 sums up to the warps).
enum { kEpiStore = 0, kEpiDot = 1, kEpiDiff = 2 };

template <int AXIS, int EPI = kEpiStore>
__global__ void __launch_bounds__(256) k_soft_pass_yz(const float *in, float *out, SoftGeom g, int mode, int R,
                                                      SoftTaps T, const float *aux = nullptr,
                                                      double *dot_out = nullptr, float scale = 0.0f) {
  extern __shared__ float slab[];   // [kSoftTileYZ + 2R][32]
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int n = AXIS == 1 ? g.H : g.D;
  const int64_t s = AXIS == 1 ? (int64_t)g.W : (int64_t)g.W * g.H;
  const int x = blockIdx.x * 32 + tx;
  const int c0 = blockIdx.y * kSoftTileYZ;
  // the other coordinate: z for the y pass, y for the z pass
  const int64_t other = AXIS == 1 ? (int64_t)blockIdx.z * g.W * g.H : (int64_t)blockIdx.z * g.W;
  const float *line = in + other + x;
  const int rows = kSoftTileYZ + 2 * R;
  for (int k = ty; k < rows; k += 8) slab[k * 32 + tx] = x < g.W ? soft_stage(line, s, c0 - R + k, n, mode) : 0.0f;
  __syncthreads();
  float hi = 0.0f, lo = 0.0f;
  if (x < g.W)
    for (int m = ty; m < kSoftTileYZ; m += 8) {
      const int c = c0 + m;
      if (c >= n) break;
      const int64_t i = other + x + (int64_t)c * s;
      const float v = soft_fold(slab + m * 32 + tx, 32, c, n, mode, R, T);
      if (EPI == kEpiDot) soft_dot_add(hi, lo, aux[i], v);
      else if (EPI == kEpiDiff) out[i] = scale * (aux[i] - v);
      else out[i] = v;
    }
  if (EPI == kEpiDot) {
    __shared__ double part[8];
    const double acc = soft_warp_dot(hi, lo);
    if (tx == 0) part[ty] = acc;
    __syncthreads();
    if (tx == 0 && ty == 0) {
      double t = 0.0;
      for (int w = 0; w < 8; w++) t += part[w];
      atomicAdd(dot_out, t);
    }
  }
}

// min / max along y (AXIS 1) or z (AXIS 2) by doubling, 32 columns x kSoftTileYZ outputs
template <int AXIS>
__global__ void __launch_bounds__(512) k_soft_ext_yz(const float *in, float *out, SoftGeom g, int is_max, int R) {
  __shared__ float slab[(kSoftTileYZ + 2 * kSoftExtMaxR) * 32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int n = AXIS == 1 ? g.H : g.D;
  const int64_t s = AXIS == 1 ? (int64_t)g.W : (int64_t)g.W * g.H;
  const int x = blockIdx.x * 32 + tx;
  const int c0 = blockIdx.y * kSoftTileYZ;
  const int64_t other = AXIS == 1 ? (int64_t)blockIdx.z * g.W * g.H : (int64_t)blockIdx.z * g.W;
  const float *line = in + other + x;
  const int rows = kSoftTileYZ + 2 * R, q_end = soft_span(R);
  for (int k = ty; k < rows; k += 16) slab[k * 32 + tx] = x < g.W ? soft_stage(line, s, c0 - R + k, n, kMin) : 0.0f;
  __syncthreads();
  for (int q = 1; q < q_end; q *= 2) {
    const int lim = rows - 2 * q + 1;
    float v[kSoftExtPer];
#pragma unroll
    for (int e = 0; e < kSoftExtPer; e++) {
      const int k = ty + 16 * e;
      v[e] = k < lim ? soft_ext(slab[k * 32 + tx], slab[(k + q) * 32 + tx], is_max) : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < kSoftExtPer; e++)
      if (ty + 16 * e < lim) slab[(ty + 16 * e) * 32 + tx] = v[e];
    __syncthreads();
  }
  if (x >= g.W) return;
  for (int m = ty; m < kSoftTileYZ; m += 16) {
    const int c = c0 + m;
    if (c >= n) break;
    out[other + x + (int64_t)c * s] = soft_ext(slab[m * 32 + tx], slab[(m + 2 * R + 1 - q_end) * 32 + tx], is_max);
  }
}

// The two transposed passes from the same tiles, again with the old operations in the old
// order: the box mean's gather (kAdjBox; the tile holds g_out, zero outside the line), and
// the min / max scatter to each window's first extreme (kAdjMin / kAdjMax; the tile holds
// the filter's input, clamped).  Window positions outside the line are clamped exactly as
// in k_soft_box_adj / k_soft_minmax_adj.
enum { kAdjBox = 0, kAdjMin = 1, kAdjMax = 2 };

__device__ __forceinline__ void soft_adj_one(const float *w, int step, int c, int n, int R, int adj, int64_t base,
                                             int64_t s, const float *g_out, float *g_in) {
  // w[k * step] is the staged value at line position c - R + k
  if (adj == kAdjBox) {
    float acc = 0.0f;
    for (int t = max(0, c - R); t <= min(n - 1, c + R); t++) acc += w[(t - c + R) * step];
    if (c == 0)
      for (int t = 0; t < min(n, R); t++) acc += (float)(R - t) * w[(t - c + R) * step];
    if (c == n - 1)
      for (int t = max(0, n - 1 - R + 1); t < n; t++) acc += (float)(t + R - (n - 1)) * w[(t - c + R) * step];
    g_in[base + (int64_t)c * s] = acc / (float)(2 * R + 1);
    return;
  }
  const float go = g_out[base + (int64_t)c * s];
  if (go == 0.0f) return;
  int arg = clampi(c - R, 0, n - 1);
  float best = w[0];
  for (int j = -R + 1; j <= R; j++) {
    const float v = w[(j + R) * step];
    if (adj == kAdjMax ? v > best : v < best) {
      best = v;
      arg = clampi(c + j, 0, n - 1);
    }
  }
  atomicAdd(g_in + base + (int64_t)arg * s, go);
}

__global__ void __launch_bounds__(kSoftTileX) k_soft_adj_x(const float *src, const float *g_out, float *g_in,
                                                           SoftGeom g, int adj, int R) {
  __shared__ float tile[kSoftRowsX][kSoftTileX + 2 * kSoftTileMaxR];
  __shared__ int at[kSoftRowsX][kSoftTileX + 2 * kSoftTileMaxR];
  const int nseg = (g.W + kSoftTileX - 1) / kSoftTileX;
  const int64_t row0 = (int64_t)(blockIdx.x / nseg) * kSoftRowsX;
  const int nr = (int)min((int64_t)kSoftRowsX, (int64_t)g.H * g.D - row0);
  const int x0 = (int)(blockIdx.x % nseg) * kSoftTileX, t = threadIdx.x;
  const int L = kSoftTileX + 2 * R;
  const int stage_mode = adj == kAdjBox ? kConv : kMin;   // zero outside / clamped
  for (int r = 0; r < nr; r++)
    for (int k = t; k < L; k += kSoftTileX) {
      tile[r][k] = soft_stage(src + (row0 + r) * g.W, 1, x0 - R + k, g.W, stage_mode);
      at[r][k] = k;
    }
  __syncthreads();
  const int x = x0 + t;
  if (adj != kAdjBox) {
    // first extreme of every window by doubling over (value, staged position) pairs
    const bool is_max = adj == kAdjMax;
    const int q_end = soft_span(R);
    for (int q = 1; q < q_end; q *= 2) {
      const int lim = L - 2 * q + 1;
      float a[kSoftRowsX][2];
      int ia[kSoftRowsX][2];
#pragma unroll
      for (int r = 0; r < kSoftRowsX; r++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int k = t + h * kSoftTileX;
          a[r][h] = 0.0f;
          ia[r][h] = 0;
          if (r < nr && k < lim) {
            a[r][h] = tile[r][k];
            ia[r][h] = at[r][k];
            soft_ext_at(a[r][h], ia[r][h], tile[r][k + q], at[r][k + q], is_max);
          }
        }
      __syncthreads();
#pragma unroll
      for (int r = 0; r < kSoftRowsX; r++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int k = t + h * kSoftTileX;
          if (r < nr && k < lim) {
            tile[r][k] = a[r][h];
            at[r][k] = ia[r][h];
          }
        }
      __syncthreads();
    }
    if (x < g.W)
      for (int r = 0; r < nr; r++) {
        const int64_t row = (row0 + r) * g.W;
        const float go = g_out[row + x];
        if (go == 0.0f) continue;
        float v = tile[r][t];
        int iv = at[r][t];
        soft_ext_at(v, iv, tile[r][t + 2 * R + 1 - q_end], at[r][t + 2 * R + 1 - q_end], is_max);
        atomicAdd(g_in + row + clampi(x0 - R + iv, 0, g.W - 1), go);
      }
    return;
  }
  if (x < g.W)
    for (int r = 0; r < nr; r++) soft_adj_one(tile[r] + t, 1, x, g.W, R, adj, (row0 + r) * g.W, 1, g_out, g_in);
}

template <int AXIS>
__global__ void __launch_bounds__(256) k_soft_adj_yz(const float *src, const float *g_out, float *g_in, SoftGeom g,
                                                     int adj, int R) {
  extern __shared__ float slab[];   // [kSoftTileYZ + 2R][32]
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int n = AXIS == 1 ? g.H : g.D;
  const int64_t s = AXIS == 1 ? (int64_t)g.W : (int64_t)g.W * g.H;
  const int x = blockIdx.x * 32 + tx;
  const int c0 = blockIdx.y * kSoftTileYZ;
  const int64_t other = AXIS == 1 ? (int64_t)blockIdx.z * g.W * g.H : (int64_t)blockIdx.z * g.W;
  const float *line = src + other + x;
  const int stage_mode = adj == kAdjBox ? kConv : kMin;
  const int rows = kSoftTileYZ + 2 * R;
  for (int k = ty; k < rows; k += 8) slab[k * 32 + tx] = x < g.W ? soft_stage(line, s, c0 - R + k, n, stage_mode) : 0.0f;
  __syncthreads();
  if (x >= g.W) return;
  for (int m = ty; m < kSoftTileYZ; m += 8) {
    const int c = c0 + m;
    if (c >= n) break;
    soft_adj_one(slab + m * 32 + tx, 32, c, n, R, adj, other + x, s, g_out, g_in);
  }
}

// the transposed min / max along y or z: each window's output gradient to its first extreme,
// found by doubling over (value, staged position) pairs; g_in must start at zero
template <int AXIS>
__global__ void __launch_bounds__(512) k_soft_ext_adj_yz(const float *src, const float *g_out, float *g_in, SoftGeom g,
                                                         int is_max, int R) {
  __shared__ float slab[(kSoftTileYZ + 2 * kSoftExtMaxR) * 32];
  __shared__ int at[(kSoftTileYZ + 2 * kSoftExtMaxR) * 32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int n = AXIS == 1 ? g.H : g.D;
  const int64_t s = AXIS == 1 ? (int64_t)g.W : (int64_t)g.W * g.H;
  const int x = blockIdx.x * 32 + tx;
  const int c0 = blockIdx.y * kSoftTileYZ;
  const int64_t other = AXIS == 1 ? (int64_t)blockIdx.z * g.W * g.H : (int64_t)blockIdx.z * g.W;
  const float *line = src + other + x;
  const int rows = kSoftTileYZ + 2 * R, q_end = soft_span(R);
  for (int k = ty; k < rows; k += 16) {
    slab[k * 32 + tx] = x < g.W ? soft_stage(line, s, c0 - R + k, n, kMin) : 0.0f;
    at[k * 32 + tx] = k;
  }
  __syncthreads();
  for (int q = 1; q < q_end; q *= 2) {
    const int lim = rows - 2 * q + 1;
    float v[kSoftExtPer];
    int iv[kSoftExtPer];
#pragma unroll
    for (int e = 0; e < kSoftExtPer; e++) {
      const int k = ty + 16 * e;
      v[e] = 0.0f;
      iv[e] = 0;
      if (k < lim) {
        v[e] = slab[k * 32 + tx];
        iv[e] = at[k * 32 + tx];
        soft_ext_at(v[e], iv[e], slab[(k + q) * 32 + tx], at[(k + q) * 32 + tx], is_max);
      }
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < kSoftExtPer; e++) {
      const int k = ty + 16 * e;
      if (k < lim) {
        slab[k * 32 + tx] = v[e];
        at[k * 32 + tx] = iv[e];
      }
    }
    __syncthreads();
  }
  if (x >= g.W) return;
  for (int m = ty; m < kSoftTileYZ; m += 16) {
    const int c = c0 + m;
    if (c >= n) break;
    const float go = g_out[other + x + (int64_t)c * s];
    if (go == 0.0f) continue;
    float a = slab[m * 32 + tx];
    int ia = at[m * 32 + tx];
    const int m2 = m + 2 * R + 1 - q_end;
    soft_ext_at(a, ia, slab[m2 * 32 + tx], at[m2 * 32 + tx], is_max);
    atomicAdd(g_in + other + x + (int64_t)clampi(c0 - R + ia, 0, n - 1) * s, go);
  }
}

// Transposed min / max pass: the output gradient of each window goes to the window's first
// extreme (the index the forward filter took it from).  g_in must start at zero.
__global__ void k_soft_minmax_adj(const float *in, const float *g_out, float *g_in, SoftGeom g, int axis, int r,
                                  int is_max, int64_t N) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const float go = g_out[i];
  if (go == 0.0f) return;
  int c, n;
  int64_t s;
  soft_axis(g, axis, i, c, s, n);
  const int64_t base = i - (int64_t)c * s;
  int arg = clampi(c - r, 0, n - 1);
  float best = in[base + (int64_t)arg * s];
  for (int j = -r + 1; j <= r; j++) {
    const int p = clampi(c + j, 0, n - 1);
    const float v = in[base + (int64_t)p * s];
    if (is_max ? v > best : v < best) {
      best = v;
      arg = p;
    }
  }
  atomicAdd(g_in + base + (int64_t)arg * s, go);
}

// Transposed box mean (nearest border), as a gather: input i receives every output t within
// r of it, and an edge input additionally receives each output whose window ran past that
// edge once per clamped tap.
__global__ void k_soft_box_adj(const float *g_out, float *g_in, SoftGeom g, int axis, int r, int64_t N) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int c, n;
  int64_t s;
  soft_axis(g, axis, i, c, s, n);
  const float *line = g_out + (i - (int64_t)c * s);
  float acc = 0.0f;
  for (int t = max(0, c - r); t <= min(n - 1, c + r); t++) acc += line[(int64_t)t * s];
  if (c == 0)
    for (int t = 0; t < min(n, r); t++) acc += (float)(r - t) * line[(int64_t)t * s];
  if (c == n - 1)
    for (int t = max(0, n - 1 - r + 1); t < n; t++) acc += (float)(t + r - (n - 1)) * line[(int64_t)t * s];
  g_in[i] = acc / (float)(2 * r + 1);
}

__global__ void k_soft_norm(const float *I, const float *e, const float *d, float *norm, float min_intensity, int64_t N) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  norm[i] = I[i] >= min_intensity ? (I[i] - e[i]) / (d[i] - e[i]) : 0.0f;
}

// Quotient rule of the normalization: g_I (direct term, written), g_e, g_d.
__global__ void k_soft_norm_adj(const float *I, const float *e, const float *d, const float *g_norm, float *g_I,
                                float *g_e, float *g_d, float min_intensity, int64_t N) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const float g = g_norm[i];
  if (I[i] >= min_intensity) {
    const float den = d[i] - e[i], inv = 1.0f / den, inv2 = inv * inv;
    g_I[i] = g * inv;
    g_e[i] = g * (I[i] - d[i]) * inv2;
    g_d[i] = -g * (I[i] - e[i]) * inv2;
  } else {
    g_I[i] = 0.0f;
    g_e[i] = 0.0f;
    g_d[i] = 0.0f;
  }
}

// out = scale * (a - b)
__global__ void k_soft_add(float *a, const float *b, int64_t N) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) a[i] += b[i];
}

// sum_i a[i] * b[i] into *out (a double, which must start at zero; compensated float32 sums
// up to the warps)
__global__ void k_soft_dot(const float *a, const float *b, int64_t N, double *out) {
  __shared__ double part[8];
  float hi = 0.0f, lo = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    soft_dot_add(hi, lo, a[i], b[i]);
  const double acc = soft_warp_dot(hi, lo);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += part[w];
    atomicAdd(out, t);
  }
}

// ---- Hessian at a point and its adjoint (element order xx, xy, xz, yy, yz, zz)
__device__ __forceinline__ int h_inner(int e) { return e < 3 ? 0 : (e < 5 ? 1 : 2); }   // xx xy xz | yy yz | zz
__device__ __forceinline__ int h_outer(int e) { return e == 0 ? 0 : (e == 1 || e == 3 ? 1 : 2); }

// Offsets of the three relaxed minor tests (kernel parameter).
struct SoftThresh {
  float v[3];
};

struct SoftPoint {
  int x, y, z;
};
__device__ __forceinline__ bool soft_in(const SoftGeom &g, int x, int y, int z) {
  return x >= 0 && y >= 0 && z >= 0 && x < g.W && y < g.H && z < g.D;
}
__device__ __forceinline__ void soft_step(int axis, int s, int &x, int &y, int &z) {
  if (axis == 0) x += s;
  else if (axis == 1) y += s;
  else z += s;
}
__device__ __forceinline__ float soft_f(const float *f, const SoftGeom &g, int x, int y, int z) {
  return soft_in(g, x, y, z) ? f[((int64_t)z * g.H + y) * g.W + x] : 0.0f;
}

__device__ void soft_hessian(const float *f, const SoftGeom &g, SoftPoint p, float h[6]) {
  for (int e = 0; e < 6; e++) {
    float v = 0.0f;
    for (int sb = -1; sb <= 1; sb += 2) {
      int qx = p.x, qy = p.y, qz = p.z;
      soft_step(h_outer(e), sb, qx, qy, qz);
      if (!soft_in(g, qx, qy, qz)) continue;   // a first derivative outside the volume is 0
      int ax = qx, ay = qy, az = qz, bx = qx, by = qy, bz = qz;
      soft_step(h_inner(e), 1, ax, ay, az);
      soft_step(h_inner(e), -1, bx, by, bz);
      const float ga = 0.5f * (soft_f(f, g, ax, ay, az) - soft_f(f, g, bx, by, bz));
      v += sb > 0 ? ga : -ga;
    }
    h[e] = 0.5f * v;
  }
}

__device__ void soft_hessian_adj(float *gf, const SoftGeom &g, SoftPoint p, const float gh[6]) {
  for (int e = 0; e < 6; e++) {
    for (int sb = -1; sb <= 1; sb += 2) {
      int qx = p.x, qy = p.y, qz = p.z;
      soft_step(h_outer(e), sb, qx, qy, qz);
      if (!soft_in(g, qx, qy, qz)) continue;
      const float c = 0.25f * (float)sb * gh[e];
      int ax = qx, ay = qy, az = qz, bx = qx, by = qy, bz = qz;
      soft_step(h_inner(e), 1, ax, ay, az);
      soft_step(h_inner(e), -1, bx, by, bz);
      if (soft_in(g, ax, ay, az)) atomicAdd(gf + ((int64_t)az * g.H + ay) * g.W + ax, c);
      if (soft_in(g, bx, by, bz)) atomicAdd(gf + ((int64_t)bz * g.H + by) * g.W + bx, -c);
    }
  }
}

__device__ __forceinline__ float sigm(float v) { return 1.0f / (1.0f + expf(-v)); }

// Score of Hessian h: sigmoid((b0 - xx) / tau) sigmoid((m2 - b1) / tau^2) sigmoid((b2 - det) /
// tau^3) with thresholds b (all zero: the reference's test xx < 0, m2 > 0, det < 0).  When
// ds is given, its derivative in h; when db is given, its derivative in b.
__device__ float soft_score(const float h[6], float tau, const float b[3], float *ds, float *db) {
  const float xx = h[0], xy = h[1], xz = h[2], yy = h[3], yz = h[4], zz = h[5];
  const float t2 = tau * tau, t3 = t2 * tau;
  const float m2 = xx * yy - xy * xy;
  const float det = xx * yy * zz + 2.0f * xy * yz * xz - xx * yz * yz - yy * xz * xz - zz * xy * xy;
  const float A = sigm((b[0] - xx) / tau), B = sigm((m2 - b[1]) / t2), C = sigm((b[2] - det) / t3);
  const float s = A * B * C;
  const float ca = -(1.0f - A) / tau, cb = (1.0f - B) / t2, cc = -(1.0f - C) / t3;
  if (ds) {
    // d det / d (xx, xy, xz, yy, yz, zz)
    const float dd[6] = {yy * zz - yz * yz, 2.0f * yz * xz - 2.0f * zz * xy, 2.0f * xy * yz - 2.0f * yy * xz,
                         xx * zz - xz * xz, 2.0f * xy * xz - 2.0f * xx * yz, xx * yy - xy * xy};
    const float dm2[6] = {yy, -2.0f * xy, 0.0f, xx, 0.0f, 0.0f};
    for (int k = 0; k < 6; k++) ds[k] = s * ((k == 0 ? ca : 0.0f) + cb * dm2[k] + cc * dd[k]);
  }
  if (db) {
    db[0] = -s * ca;
    db[1] = -s * cb;
    db[2] = -s * cc;
  }
  return s;
}

// Forward at the points: scores (optional) and the loss (double, out must start at zero).
__global__ void k_soft_points(const float *dog, SoftGeom g, const int32_t *pos, int n_pos, const int32_t *neg,
                              int n_neg, float tau, SoftThresh b, float *scores, double *loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pos + n_neg) return;
  const int32_t *q = i < n_pos ? pos + 3 * i : neg + 3 * (i - n_pos);
  const SoftPoint p{q[2], q[1], q[0]};
  float h[6];
  soft_hessian(dog, g, p, h);
  const float s = soft_score(h, tau, b.v, nullptr, nullptr);
  if (scores) scores[i] = s;
  atomicAdd(loss, i < n_pos ? (double)s / n_pos : -(double)s / n_neg);
}

// Backward at the points: d loss / d dog scattered into gdog (which must start at zero), and
// d loss / d thresholds summed into gb[0..2] (double, zeroed first) when gb is given.
__global__ void k_soft_points_adj(const float *dog, SoftGeom g, const int32_t *pos, int n_pos, const int32_t *neg,
                                  int n_neg, float tau, SoftThresh b, float grad_loss, float *gdog, double *gb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pos + n_neg) return;
  const int32_t *q = i < n_pos ? pos + 3 * i : neg + 3 * (i - n_pos);
  const SoftPoint p{q[2], q[1], q[0]};
  float h[6], ds[6], db[3];
  soft_hessian(dog, g, p, h);
  soft_score(h, tau, b.v, ds, db);
  const float w = i < n_pos ? grad_loss / (float)n_pos : -grad_loss / (float)n_neg;
  for (int k = 0; k < 6; k++) ds[k] *= w;
  soft_hessian_adj(gdog, g, p, ds);
  if (gb)
    for (int k = 0; k < 3; k++) atomicAdd(gb + k, (double)db[k] * (double)w);
}

__global__ void k_soft_to_float(const double *in, float *out, int n) {
  const int i = threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

// ------------------------------------------------------------------ host side
namespace {

struct SoftRun {
  const hdog_soft_params &p;
  SoftGeom g;
  int64_t N;
  cudaStream_t st;
  float *w;      // workspace slots of N floats (after the accumulators)
  double *acc;   // 16 doubles at the start of the workspace
  unsigned blocks() const { return ceil_div(N, 256); }
  float *slot(int k) const { return w + (int64_t)k * N; }
};

enum { S_MN1, S_MN2, S_MN, S_MX1, S_MX2, S_MX, S_E, S_D, S_NORM, S_DOG, S_T1, S_T2, S_T3, S_GDOG, S_GA, S_GB, S_GC,
       kSoftSlots };

SoftTaps no_taps() {
  SoftTaps t;
  memset(&t, 0, sizeof(t));
  return t;
}

// Normalized Gaussian taps of sigma (or their derivative in sigma), radius (int)(2 sigma + 0.5).
SoftTaps gauss_taps_f(double sigma, bool derivative) {
  SoftTaps t = no_taps();
  const int r = (int)(2.0 * sigma + 0.5);
  t.r = r;
  double e[kSoftMaxTaps], sum = 0.0, m2 = 0.0;
  for (int k = -r; k <= r; k++) {
    e[k + r] = exp(-0.5 * k * k / (sigma * sigma));
    sum += e[k + r];
  }
  for (int k = -r; k <= r; k++) m2 += e[k + r] / sum * (double)k * k;
  for (int k = -r; k <= r; k++) {
    const double tk = e[k + r] / sum;
    t.k[k + r] = (float)(derivative ? tk * ((double)k * k - m2) / (sigma * sigma * sigma) : tk);
  }
  return t;
}

void pass(const SoftRun &R, const float *in, float *out, int axis, int mode, int r, const SoftTaps &T) {
  const int reach = mode == kConv ? T.r : r;
  const SoftGeom &g = R.g;
  if (reach > kSoftTileMaxR) {
    KLAUNCH("k_soft_pass", R.st, (k_soft_pass<<<R.blocks(), 256, 0, R.st>>>(in, out, g, axis, mode, r, T, R.N)));
    return;
  }
  if (axis == 0) {
    const unsigned blocks = (unsigned)(ceil_div(g.W, kSoftTileX) * ceil_div((int64_t)g.H * g.D, kSoftRowsX));
    KLAUNCH("k_soft_pass_x", R.st, (k_soft_pass_x<<<blocks, kSoftTileX, 0, R.st>>>(in, out, g, mode, reach, T)));
    return;
  }
  const size_t smem = (size_t)(kSoftTileYZ + 2 * reach) * 32 * sizeof(float);
  const int n = axis == 1 ? g.H : g.D, other = axis == 1 ? g.D : g.H;
  const dim3 grid((unsigned)ceil_div(g.W, 32), (unsigned)ceil_div(n, kSoftTileYZ), (unsigned)other);
  if ((mode == kMin || mode == kMax) && reach <= kSoftExtMaxR) {
    if (axis == 1)
      KLAUNCH("k_soft_ext_y", R.st, (k_soft_ext_yz<1><<<grid, dim3(32, 16), 0, R.st>>>(in, out, g, mode == kMax, reach)));
    else
      KLAUNCH("k_soft_ext_z", R.st, (k_soft_ext_yz<2><<<grid, dim3(32, 16), 0, R.st>>>(in, out, g, mode == kMax, reach)));
    return;
  }
  if (axis == 1)
    KLAUNCH("k_soft_pass_y", R.st, (k_soft_pass_yz<1><<<grid, dim3(32, 8), smem, R.st>>>(in, out, g, mode, reach, T)));
  else
    KLAUNCH("k_soft_pass_z", R.st, (k_soft_pass_yz<2><<<grid, dim3(32, 8), smem, R.st>>>(in, out, g, mode, reach, T)));
}

// the correlation along z with T, summed against w into *acc (double) instead of stored
void pass_z_dot(const SoftRun &R, const float *in, const SoftTaps &T, const float *w, double *acc) {
  static_assert(kSoftMaxRadius <= kSoftTileMaxR, "Gaussian taps fit the z tile");
  const SoftGeom &g = R.g;
  const size_t smem = (size_t)(kSoftTileYZ + 2 * T.r) * 32 * sizeof(float);
  const dim3 grid((unsigned)ceil_div(g.W, 32), (unsigned)ceil_div(g.D, kSoftTileYZ), (unsigned)g.H);
  KLAUNCH("k_soft_pass_z_dot", R.st, (k_soft_pass_yz<2, kEpiDot><<<grid, dim3(32, 8), smem, R.st>>>(
                                         in, nullptr, g, kConv, T.r, T, w, acc)));
}

// the separable Gaussian (x, y, then z) with the DoG difference folded into the z pass:
// out = scale * (sub - in * G), the same operations as a separate difference kernel
void conv3_diff(const SoftRun &R, const float *in, float *out, const SoftTaps &tx, const SoftTaps &ty,
                const SoftTaps &tz, float *t1, float *t2, const float *sub, float scale) {
  pass(R, in, t1, 0, kConv, 0, tx);
  pass(R, t1, t2, 1, kConv, 0, ty);
  const SoftGeom &g = R.g;
  const size_t smem = (size_t)(kSoftTileYZ + 2 * tz.r) * 32 * sizeof(float);
  const dim3 grid((unsigned)ceil_div(g.W, 32), (unsigned)ceil_div(g.D, kSoftTileYZ), (unsigned)g.H);
  KLAUNCH("k_soft_pass_z_diff", R.st, (k_soft_pass_yz<2, kEpiDiff><<<grid, dim3(32, 8), smem, R.st>>>(
                                          t2, out, g, kConv, tz.r, tz, sub, nullptr, scale)));
}

// a transposed pass along `axis`: box gather (src = g_out, into g_in) or min / max scatter
// (src = the filter's input, g_out into the zeroed g_in)
void adj_pass(const SoftRun &R, const float *src, const float *g_out, float *g_in, int axis, int adj, int r) {
  const SoftGeom &g = R.g;
  const unsigned nb = R.blocks();
  if (r > kSoftTileMaxR) {
    if (adj == kAdjBox)
      KLAUNCH("k_soft_box_adj", R.st, (k_soft_box_adj<<<nb, 256, 0, R.st>>>(src, g_in, g, axis, r, R.N)));
    else
      KLAUNCH("k_soft_minmax_adj", R.st, (k_soft_minmax_adj<<<nb, 256, 0, R.st>>>(src, g_out, g_in, g, axis, r,
                                                                                 adj == kAdjMax, R.N)));
    return;
  }
  if (axis == 0) {
    const unsigned blocks = (unsigned)(ceil_div(g.W, kSoftTileX) * ceil_div((int64_t)g.H * g.D, kSoftRowsX));
    KLAUNCH("k_soft_adj_x", R.st, (k_soft_adj_x<<<blocks, kSoftTileX, 0, R.st>>>(src, g_out, g_in, g, adj, r)));
    return;
  }
  const int n = axis == 1 ? g.H : g.D, other = axis == 1 ? g.D : g.H;
  if (adj != kAdjBox && r <= kSoftExtMaxR) {
    const dim3 grid((unsigned)ceil_div(g.W, 32), (unsigned)ceil_div(n, kSoftTileYZ), (unsigned)other);
    if (axis == 1)
      KLAUNCH("k_soft_ext_adj_y", R.st, (k_soft_ext_adj_yz<1><<<grid, dim3(32, 16), 0, R.st>>>(src, g_out, g_in, g,
                                                                                              adj == kAdjMax, r)));
    else
      KLAUNCH("k_soft_ext_adj_z", R.st, (k_soft_ext_adj_yz<2><<<grid, dim3(32, 16), 0, R.st>>>(src, g_out, g_in, g,
                                                                                              adj == kAdjMax, r)));
    return;
  }
  const size_t smem = (size_t)(kSoftTileYZ + 2 * r) * 32 * sizeof(float);
  const dim3 grid((unsigned)ceil_div(g.W, 32), (unsigned)ceil_div(n, kSoftTileYZ), (unsigned)other);
  if (axis == 1)
    KLAUNCH("k_soft_adj_y", R.st, (k_soft_adj_yz<1><<<grid, dim3(32, 8), smem, R.st>>>(src, g_out, g_in, g, adj, r)));
  else
    KLAUNCH("k_soft_adj_z", R.st, (k_soft_adj_yz<2><<<grid, dim3(32, 8), smem, R.st>>>(src, g_out, g_in, g, adj, r)));
}

// conv of `in` with taps (tx, ty, tz) along x, y, z -> out (t1, t2 as temporaries)
void conv3(const SoftRun &R, const float *in, float *out, const SoftTaps &tx, const SoftTaps &ty, const SoftTaps &tz,
           float *t1, float *t2) {
  pass(R, in, t1, 0, kConv, 0, tx);
  pass(R, t1, t2, 1, kConv, 0, ty);
  pass(R, t2, out, 2, kConv, 0, tz);
}

// The forward chain into the workspace: min/max chains, box means, norm, dog.
void forward_chain(const SoftRun &R, const float *vol) {
  const hdog_soft_params &p = R.p;
  const SoftTaps none = no_taps();
  const int rr[3] = {p.radius_norm_xy, p.radius_norm_xy, p.radius_norm_z};
  const float *src_mn = vol, *src_mx = vol;
  const int smn[3] = {S_MN1, S_MN2, S_MN}, smx[3] = {S_MX1, S_MX2, S_MX};
  for (int a = 0; a < 3; a++) {
    pass(R, src_mn, R.slot(smn[a]), a, kMin, rr[a], none);
    pass(R, src_mx, R.slot(smx[a]), a, kMax, rr[a], none);
    src_mn = R.slot(smn[a]);
    src_mx = R.slot(smx[a]);
  }
  pass(R, R.slot(S_MN), R.slot(S_T1), 0, kBox, rr[0], none);
  pass(R, R.slot(S_T1), R.slot(S_T2), 1, kBox, rr[1], none);
  pass(R, R.slot(S_T2), R.slot(S_E), 2, kBox, rr[2], none);
  pass(R, R.slot(S_MX), R.slot(S_T1), 0, kBox, rr[0], none);
  pass(R, R.slot(S_T1), R.slot(S_T2), 1, kBox, rr[1], none);
  pass(R, R.slot(S_T2), R.slot(S_D), 2, kBox, rr[2], none);
  KLAUNCH("k_soft_norm", R.st, (k_soft_norm<<<R.blocks(), 256, 0, R.st>>>(vol, R.slot(S_E), R.slot(S_D), R.slot(S_NORM),
                                                                        p.min_intensity, R.N)));
  const float *s = p.sigma;
  conv3(R, R.slot(S_NORM), R.slot(S_T3), gauss_taps_f(s[0], false), gauss_taps_f(s[1], false), gauss_taps_f(s[2], false),
        R.slot(S_T1), R.slot(S_T2));
  const float nrm = (float)pow((double)s[0] * s[1] * s[2], (double)p.gamma);
  conv3_diff(R, R.slot(S_NORM), R.slot(S_DOG), gauss_taps_f(s[3], false), gauss_taps_f(s[4], false),
             gauss_taps_f(s[5], false), R.slot(S_T1), R.slot(S_T2), R.slot(S_T3), nrm);
}

SoftThresh thresh_of(const hdog_soft_params &p) {
  SoftThresh b;
  for (int k = 0; k < 3; k++) b.v[k] = p.thresh[k];
  return b;
}

int check_params(const hdog_soft_params *p, const float *vol, const int32_t *pos, int n_pos, const int32_t *neg,
                 int n_neg, void *work) {
  if (!p || !vol || !work || n_pos < 0 || n_neg < 0 || (n_pos && !pos) || (n_neg && !neg))
    return HDOG_ERR_ARG;
  if (p->width < 1 || p->height < 1 || p->depth < 1 || p->radius_norm_xy < 0 || p->radius_norm_z < 0 ||
      p->radius_norm_xy > 1000 || p->radius_norm_z > 1000 || !(p->tau > 0.0f))
    return HDOG_ERR_PARAM;
  for (int k = 0; k < 6; k++)
    if (!(p->sigma[k] > 0.0f) || (int)(2.0 * p->sigma[k] + 0.5) > kSoftMaxRadius) return HDOG_ERR_SHAPE;
  return HDOG_OK;
}

}  // namespace

size_t soft_workspace_bytes(const hdog_soft_params &p) {
  return 16 * sizeof(double) + (size_t)kSoftSlots * p.width * p.height * p.depth * sizeof(float);
}

int soft_forward(const hdog_soft_params *p, const float *vol, const int32_t *pos, int n_pos, const int32_t *neg,
                 int n_neg, float *loss, float *scores, void *work, cudaStream_t st) {
  const int rc = check_params(p, vol, pos, n_pos, neg, n_neg, work);
  if (rc != HDOG_OK || !loss) return rc != HDOG_OK ? rc : HDOG_ERR_ARG;
  SoftRun R{*p, SoftGeom{p->width, p->height, p->depth}, (int64_t)p->width * p->height * p->depth, st,
            static_cast<float *>(work), nullptr};
  R.acc = static_cast<double *>(work);
  R.w = reinterpret_cast<float *>(R.acc + 16);
  forward_chain(R, vol);
  cudaMemsetAsync(R.acc, 0, sizeof(double), st);
  if (n_pos + n_neg > 0)
    KLAUNCH("k_soft_points", st, (k_soft_points<<<ceil_div(n_pos + n_neg, 128), 128, 0, st>>>(
                                     R.slot(S_DOG), R.g, pos, n_pos, neg, n_neg, p->tau, thresh_of(*p), scores,
                                     R.acc)));
  k_soft_to_float<<<1, 32, 0, st>>>(R.acc, loss, 1);
  return HDOG_OK;
}

int soft_backward(const hdog_soft_params *p, const float *vol, const int32_t *pos, int n_pos, const int32_t *neg,
                  int n_neg, float grad_loss, float *grad_vol, float *grad_sigma, float *grad_thresh, void *work,
                  cudaStream_t st, bool forward_kept) {
  const int rc = check_params(p, vol, pos, n_pos, neg, n_neg, work);
  if (rc != HDOG_OK) return rc;
  SoftRun R{*p, SoftGeom{p->width, p->height, p->depth}, (int64_t)p->width * p->height * p->depth, st,
            static_cast<float *>(work), nullptr};
  R.acc = static_cast<double *>(work);
  R.w = reinterpret_cast<float *>(R.acc + 16);
  const unsigned nb = R.blocks();
  // The backward reads the forward chain's slots (S_MN1 .. S_DOG) and writes only the others,
  // so a workspace that soft_forward filled for the same inputs still holds them.
  if (!forward_kept) forward_chain(R, vol);
  float *gdog = R.slot(S_GDOG);
  cudaMemsetAsync(gdog, 0, R.N * sizeof(float), st);
  double *gb = R.acc + 8;   // threshold gradients
  cudaMemsetAsync(gb, 0, 3 * sizeof(double), st);
  if (n_pos + n_neg > 0)
    KLAUNCH("k_soft_points_adj", st, (k_soft_points_adj<<<ceil_div(n_pos + n_neg, 128), 128, 0, st>>>(
                                         R.slot(S_DOG), R.g, pos, n_pos, neg, n_neg, p->tau, thresh_of(*p), grad_loss,
                                         gdog, gb)));
  if (grad_thresh) k_soft_to_float<<<1, 32, 0, st>>>(gb, grad_thresh, 3);
  const float *s = p->sigma;
  const float nrm = (float)pow((double)s[0] * s[1] * s[2], (double)p->gamma);
  if (grad_sigma) {
    // acc[0..5]: <gdog, d dog / d sigma_k> without the normalizer term; acc[6]: <gdog, dog>
    cudaMemsetAsync(R.acc, 0, 8 * sizeof(double), st);
    const unsigned db = 152 * 4;
    // Per scale: <gdog, C_z C_y C_x norm> with the derivative taps on one axis.  The plain x
    // pass serves the y and z derivatives, and every z pass folds straight into the dot.
    float *nm = R.slot(S_NORM), *t1 = R.slot(S_T1), *t2 = R.slot(S_T2);
    for (int sc = 0; sc < 2; sc++) {
      SoftTaps pl[3], dv[3];
      for (int a = 0; a < 3; a++) {
        pl[a] = gauss_taps_f(s[3 * sc + a], false);
        dv[a] = gauss_taps_f(s[3 * sc + a], true);
      }
      double *acc = R.acc + 3 * sc;
      pass(R, nm, t1, 0, kConv, 0, pl[0]);
      pass(R, t1, t2, 1, kConv, 0, pl[1]);
      pass_z_dot(R, t2, dv[2], gdog, acc + 2);
      pass(R, t1, t2, 1, kConv, 0, dv[1]);
      pass_z_dot(R, t2, pl[2], gdog, acc + 1);
      pass(R, nm, t1, 0, kConv, 0, dv[0]);
      pass(R, t1, t2, 1, kConv, 0, pl[1]);
      pass_z_dot(R, t2, pl[2], gdog, acc + 0);
    }
    KLAUNCH("k_soft_dot", st, (k_soft_dot<<<db, 256, 0, st>>>(gdog, R.slot(S_DOG), R.N, R.acc + 6)));
    double h[8];
    HDOG_CUDA_TRY(cudaMemcpyAsync(h, R.acc, sizeof(h), cudaMemcpyDeviceToHost, st));
    HDOG_CUDA_TRY(cudaStreamSynchronize(st));
    float gs[6];
    for (int k = 0; k < 6; k++) {
      double v = (k < 3 ? nrm : -nrm) * h[k];
      if (k < 3) v += (double)p->gamma / s[k] * h[6];   // d normalizer / d sigma = gamma normalizer / sigma
      gs[k] = (float)v;
    }
    HDOG_CUDA_TRY(cudaMemcpyAsync(grad_sigma, gs, sizeof(gs), cudaMemcpyHostToDevice, st));
    HDOG_CUDA_TRY(cudaStreamSynchronize(st));
  }
  if (grad_vol) {
    // g_norm = normalizer (G1 - G2)^T gdog = normalizer (G1 gdog - G2 gdog)
    conv3(R, gdog, R.slot(S_T3), gauss_taps_f(s[0], false), gauss_taps_f(s[1], false), gauss_taps_f(s[2], false),
          R.slot(S_T1), R.slot(S_T2));
    conv3_diff(R, gdog, R.slot(S_GB), gauss_taps_f(s[3], false), gauss_taps_f(s[4], false), gauss_taps_f(s[5], false),
               R.slot(S_T1), R.slot(S_T2), R.slot(S_T3), nrm);
    // quotient rule: direct term into grad_vol, g_e -> S_T1, g_d -> S_T2
    KLAUNCH("k_soft_norm_adj", st, (k_soft_norm_adj<<<nb, 256, 0, st>>>(vol, R.slot(S_E), R.slot(S_D), R.slot(S_GB),
                                                                       grad_vol, R.slot(S_T1), R.slot(S_T2),
                                                                       p->min_intensity, R.N)));
    const int rr[3] = {p->radius_norm_xy, p->radius_norm_xy, p->radius_norm_z};
    // min side then max side: box means transposed z -> y -> x, then the min / max filters
    // transposed z -> y -> x, each scattering into a zeroed buffer but the last, which
    // scatters straight into the input gradient (holding the quotient rule's direct term)
    int last = -1;   // the axis of the last min / max pass: the lowest one with a window
    for (int a = 2; a >= 0; a--)
      if (rr[a] != 0) last = a;
    for (int side = 0; side < 2; side++) {
      float *g = R.slot(side == 0 ? S_T1 : S_T2);
      float *ping = R.slot(S_GA), *pong = R.slot(S_GC);
      const float *cur = g;
      for (int a = 2; a >= 0; a--) {
        float *dst = (cur == ping) ? pong : ping;
        if (rr[a] == 0) continue;
        adj_pass(R, cur, nullptr, dst, a, kAdjBox, rr[a]);
        cur = dst;
      }
      // filter inputs of the forward passes x, y, z: vol, *1, *2
      const float *fin[3] = {vol, R.slot(side == 0 ? S_MN1 : S_MX1), R.slot(side == 0 ? S_MN2 : S_MX2)};
      for (int a = 2; a >= 0; a--) {
        if (rr[a] == 0) continue;
        float *dst = grad_vol;
        if (a != last) {
          dst = (cur == ping) ? pong : ping;
          if (dst == g) dst = R.slot(S_GB);
          cudaMemsetAsync(dst, 0, R.N * sizeof(float), st);
        }
        adj_pass(R, fin[a], cur, dst, a, side == 0 ? kAdjMin : kAdjMax, rr[a]);
        cur = dst;
      }
      if (last < 0) KLAUNCH("k_soft_add", st, (k_soft_add<<<nb, 256, 0, st>>>(grad_vol, cur, R.N)));
    }
  }
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

}  // namespace hdog
