// norm.cu -- intensity normalization and the regional-erosion operator, sm_103a.
//
// Reference: src/3D/NormalizeFilter.cu (Normalize3DFilter :603-654) and
// src/3D/Erosion3DFilter.cu (Erosion3DFilter :260-268).
//
//   ero  = min over a (2rxy+1)^2 (2rz+1) box, dil = max over it    (nearest border)
//   ero_l = box mean of ero, dil_l = box mean of dil                 (nearest border)
//   norm = I >= min_intensity ? (I - ero_l) / (dil_l - ero_l) : 0
//
// Min and max are exact, so they run in whatever order is cheapest; the box means must
// round exactly like the reference, whose passes go x -> y -> z and each is the
// sequential float sum `val = 0; for j in 0..2r: val += s[j]` times 1.0f/(2r+1).
// Five passes, each one read and one write of the volume:
//
//   mm_z      uint16 -> packed u32     z window, four columns per thread
//   mm_y      u32 -> u32               van Herk / Gil-Werman column window in smem
//   mm_x_box  u32 -> float2            van Herk / Gil-Werman row window, then the x box
//                                      sum as exact integer sliding sums (2r+1 <= 256:
//                                      every partial sum of the reference's float chain
//                                      is an integer below 2^24, hence exact)
//   box_y     float2 -> float2         the literal y chain, erosion and dilation side by
//                                      side, K outputs per thread from a register window
//   box_z_norm float2 + uint16 -> float the literal z chain fused with the normalization
//
// Erosion and dilation travel as one packed u32 per voxel: low half the running min,
// high half 65535 minus the running max, so one __vminu2 combines both.
#include "kernels.cuh"

namespace hdog {

// pack_mm(0, 0): the value a zero-border position contributes
constexpr uint32_t kZeroPacked = 0xFFFF0000u;

// ---------------------------------------------------------------- z pass (min/max)
// VEC consecutive positions of the slice plane per thread (VEC 4: one 8-byte load of
// four uint16 per slice).  Slices at or past depth_valid read as zero (the zero tail
// HDoG3D_main.cpp:166-169 writes for a short last substack).  BORDER: 0 nearest
// (normalization), 1 zero (erosion operator).
template <int BORDER, int VEC>
__global__ void __launch_bounds__(256) k_mm_z(const Sub *subs, int rz, uint32_t *mm) {
  const Sub S = subs[blockIdx.y];
  const int64_t plane = (int64_t)S.W * S.H;
  const int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * VEC;
  if (p >= plane) return;
  const int D = S.D, dv = S.depth_valid;
  const uint16_t *src = S.src + p;
  uint32_t *out = mm + S.vox + p;
  for (int z = 0; z < D; z++) {
    int lo = z - rz, hi = z + rz;
    // nearest border repeats the edge slice (no new value); a zero border, or a slice
    // of the zero tail inside the window, adds a 0
    bool zero = BORDER == 1 && (lo < 0 || hi >= D);
    lo = max(lo, 0);
    hi = min(hi, D - 1);
    if (hi >= dv) zero = true;
    hi = min(hi, dv - 1);
    const uint16_t *q = src + (int64_t)lo * plane;
    if (VEC == 4) {
      uint32_t mn0 = 0xFFFFFFFFu, mn1 = 0xFFFFFFFFu, mx0 = 0u, mx1 = 0u;
      for (int zz = lo; zz <= hi; zz++, q += plane) {
        const uint2 v = __ldg(reinterpret_cast<const uint2 *>(q));
        mn0 = __vminu2(mn0, v.x);
        mx0 = __vmaxu2(mx0, v.x);
        mn1 = __vminu2(mn1, v.y);
        mx1 = __vmaxu2(mx1, v.y);
      }
      if (zero) { mn0 = 0u; mn1 = 0u; }
      const uint32_t n0 = ~mx0, n1 = ~mx1;
      uint4 o;
      o.x = __byte_perm(mn0, n0, 0x5410);
      o.y = __byte_perm(mn0, n0, 0x7632);
      o.z = __byte_perm(mn1, n1, 0x5410);
      o.w = __byte_perm(mn1, n1, 0x7632);
      *reinterpret_cast<uint4 *>(out + (int64_t)z * plane) = o;
    } else {
      uint32_t mn = 0xFFFFu, mx = 0u;
      for (int zz = lo; zz <= hi; zz++, q += plane) {
        const uint32_t v = __ldg(q);
        mn = min(mn, v);
        mx = max(mx, v);
      }
      out[(int64_t)z * plane] = pack_mm(zero ? 0u : mn, mx);
    }
  }
}

// The same z pass with nearest borders and a compile-time radius, streaming van Herk /
// Gil-Werman in registers: a thread owns two neighbouring columns and runs down z, every
// input slice loaded once (the windowed loop above reads each one 2R+1 times).  Both
// voxels are packed as (v, 65535 - v), so one __vminu2 carries the min and the max.
template <int R>
__global__ void __launch_bounds__(128) k_mm_z_stream(const Sub *subs, uint32_t *mm) {
  constexpr int L = 2 * R + 1;
  const Sub S = subs[blockIdx.y];
  const int64_t plane = (int64_t)S.W * S.H;
  const int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 2;
  if (p >= plane) return;
  const int D = S.D, dv = S.depth_valid;
  const uint16_t *col = S.src + p;
  uint32_t *oc = mm + S.vox + p;
  auto ld = [&](int z) -> uint2 {
    z = clampi(z, 0, D - 1);
    if (z >= dv) return make_uint2(kZeroPacked, kZeroPacked);
    const uint32_t v = __ldg(reinterpret_cast<const uint32_t *>(col + (int64_t)z * plane));
    return make_uint2(__byte_perm(v, ~v, 0x5410), __byte_perm(v, ~v, 0x7632));
  };
  auto vmin = [](uint2 a, uint2 b) { return make_uint2(__vminu2(a.x, b.x), __vminu2(a.y, b.y)); };
  uint2 suf[L], cur[L];
#pragma unroll
  for (int j = 0; j < L; j++) suf[j] = ld(j - R);
#pragma unroll
  for (int j = L - 2; j >= 0; j--) suf[j] = vmin(suf[j], suf[j + 1]);
  for (int t0 = 0; t0 < D; t0 += L) {
#pragma unroll
    for (int j = 0; j < L; j++) cur[j] = ld(t0 - R + L + j);
    uint2 pre = make_uint2(0xFFFFFFFFu, 0xFFFFFFFFu);
#pragma unroll
    for (int i = 0; i < L; i++) {
      const uint2 m = i == 0 ? suf[0] : vmin(suf[i], pre);
      if (t0 + i < D) *reinterpret_cast<uint2 *>(oc + (int64_t)(t0 + i) * plane) = m;
      pre = vmin(pre, cur[i]);
    }
    suf[L - 1] = cur[L - 1];
#pragma unroll
    for (int j = L - 2; j >= 0; j--) suf[j] = vmin(cur[j], suf[j + 1]);
  }
}

// Van Herk / Gil-Werman over blocks of L entries of a smem line: g = running min from
// each block's start (written to G), h = running min to each block's end (written over
// A).  The window [t, t + L - 1] is then min(h[t], g[t + L - 1]).
__device__ __forceinline__ void vhgw_chain(uint32_t *A, uint32_t *G, int i0, int i1, int step) {
  uint32_t run = 0xFFFFFFFFu;
  for (int i = i0; i < i1; i++) {
    run = __vminu2(run, A[i * step]);
    G[i * step] = run;
  }
  run = 0xFFFFFFFFu;
  for (int i = i1 - 1; i >= i0; i--) {
    run = __vminu2(run, A[i * step]);
    A[i * step] = run;
  }
}

// ---------------------------------------------------------------- y pass (min/max)
// A block owns 32 columns x ty output rows of one slice; it stages rows
// [y0 - r, y0 + ty + r) (border rule applied) and runs one chain per (column, block).
template <int BORDER>
__global__ void __launch_bounds__(256) k_mm_y(const Sub *subs, int r, int ty, const uint32_t *in, uint32_t *out) {
  extern __shared__ uint32_t smy[];
  const Sub S = subs[blockIdx.y];
  const int W = S.W, H = S.H;
  const int tx_n = (W + 31) / 32, ty_n = (H + ty - 1) / ty;
  const int64_t bid = blockIdx.x;
  if (bid >= (int64_t)tx_n * ty_n * S.D) return;
  const int z = (int)(bid / ((int64_t)tx_n * ty_n));
  const int rem = (int)(bid % ((int64_t)tx_n * ty_n));
  const int x0 = (rem % tx_n) * 32, y0 = (rem / tx_n) * ty;
  const int L = 2 * r + 1, n0 = ty + 2 * r;
  uint32_t *A = smy, *G = smy + n0 * 32;
  const int c = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int x = x0 + c;
  const bool xin = x < W;
  const uint32_t *sl = in + S.vox + (int64_t)z * W * H + (xin ? x : 0);
  for (int i = w; i < n0; i += nw) {
    const int y = y0 - r + i;
    uint32_t v;
    if (BORDER == 1 && (y < 0 || y >= H)) v = kZeroPacked;
    else v = sl[(int64_t)clampi(y, 0, H - 1) * W];
    A[i * 32 + c] = v;
  }
  __syncthreads();
  const int nb = (n0 + L - 1) / L;
  for (int b = w; b < nb; b += nw) vhgw_chain(A + c, G + c, b * L, min(b * L + L, n0), 32);
  __syncthreads();
  if (!xin) return;
  uint32_t *o = out + S.vox + (int64_t)z * W * H + x;
  const int tn = min(ty, H - y0);
  for (int t = w; t < tn; t += nw) o[(int64_t)(y0 + t) * W] = __vminu2(A[t * 32 + c], G[(t + 2 * r) * 32 + c]);
}

// ---------------------------------------------------------------- x pass (min/max + box)
// A block owns ry rows x tx outputs.  MODE 0: min/max window, then the exact x box sum
// -> float2 (ero_x, dil_x); MODE 1: min window only -> uint16 (erosion result); MODE 2:
// min/max window only -> packed u32 (followed by the float-chain box for 2r+1 > 256).
constexpr int kBoxC = 16;   // box outputs per thread (sliding integer sums)

template <int BORDER, int MODE>
__global__ void __launch_bounds__(256) k_mm_x(const Sub *subs, int r, int ry, int tx, const uint32_t *in,
                                              void *out) {
  extern __shared__ uint32_t smx[];
  const Sub S = subs[blockIdx.y];
  const int W = S.W;
  const int64_t rows = (int64_t)S.H * S.D;
  const int segs = (W + tx - 1) / tx;
  const int64_t bid = blockIdx.x;
  if (bid >= ((rows + ry - 1) / ry) * segs) return;
  const int64_t row0 = (bid / segs) * ry;
  const int x0 = (int)(bid % segs) * tx;
  const int hm = MODE == 0 ? r : 0;            // halo of the min/max result the box needs
  const int n0 = tx + 2 * hm + 2 * r;          // staged entries per row
  const int stride = n0 | 1;                   // odd: chains of neighbouring rows hit distinct banks
  uint32_t *A = smx, *G = smx + ry * stride;
  const int base = x0 - hm - r;                // x of A[row][0]
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  for (int rl = w; rl < ry; rl += nw) {
    const int64_t row = min(row0 + rl, rows - 1);
    const uint32_t *line = in + S.vox + row * W;
    for (int i = lane; i < n0; i += 32) {
      const int xx = base + i;
      uint32_t v;
      if (BORDER == 1 && (xx < 0 || xx >= W)) v = kZeroPacked;
      else v = line[clampi(xx, 0, W - 1)];
      A[rl * stride + i] = v;
    }
  }
  __syncthreads();
  const int L = 2 * r + 1;
  const int nb = (n0 + L - 1) / L;
  for (int ch = tid; ch < ry * nb; ch += blockDim.x) {
    const int rl = ch % ry, b = ch / ry;
    vhgw_chain(A + rl * stride, G + rl * stride, b * L, min(b * L + L, n0), 1);
  }
  __syncthreads();
  const int tn = min(tx, W - x0);
  if (MODE != 0) {
    for (int rl = w; rl < ry; rl += nw) {
      const int64_t row = row0 + rl;
      if (row >= rows) break;
      for (int k = lane; k < tn; k += 32) {
        const uint32_t m = __vminu2(A[rl * stride + k], G[rl * stride + k + 2 * r]);
        if (MODE == 1) reinterpret_cast<uint16_t *>(out)[S.vox + row * W + x0 + k] = (uint16_t)(m & 0xFFFFu);
        else reinterpret_cast<uint32_t *>(out)[S.vox + row * W + x0 + k] = m;
      }
    }
    return;
  }
  // m at x = x0 - r + k (nearest border: positions outside the row take the edge value)
  const int nm = tx + 2 * r, mstride = nm | 1;
  uint32_t *M = G + ry * stride;
  for (int rl = w; rl < ry; rl += nw)
    for (int k = lane; k < nm; k += 32) {
      const int kc = clampi(x0 - r + k, 0, W - 1) - (x0 - r);
      M[rl * mstride + k] = __vminu2(A[rl * stride + kc], G[rl * stride + kc + 2 * r]);
    }
  __syncthreads();
  // sliding sums, C outputs per thread; results staged (over A and G) for coalesced stores
  float2 *stage = reinterpret_cast<float2 *>(smx);
  const int sstride = tx + 1;
  const float inv = 1.0f / (float)L;
  const uint32_t full = (uint32_t)L * 0xFFFFu;
  const int nchunks = tx / kBoxC;
  for (int ch = tid; ch < ry * nchunks; ch += blockDim.x) {
    const int rl = ch % ry, c0 = (ch / ry) * kBoxC;
    const uint32_t *m = M + rl * mstride + c0;
    uint32_t slo = 0, shi = 0;
    for (int j = 0; j < L; j++) {
      const uint32_t v = m[j];
      slo += v & 0xFFFFu;
      shi += v >> 16;
    }
    float2 res[kBoxC];
#pragma unroll
    for (int t = 0; t < kBoxC; t++) {
      res[t] = make_float2((float)slo * inv, (float)(full - shi) * inv);
      if (t + 1 < kBoxC) {
        const uint32_t vn = m[t + L], vo = m[t];
        slo += (vn & 0xFFFFu) - (vo & 0xFFFFu);
        shi += (vn >> 16) - (vo >> 16);
      }
    }
    // A and G are free once M is built: the stage overwrites them while M is still read
#pragma unroll
    for (int t = 0; t < kBoxC; t++) stage[rl * sstride + c0 + t] = res[t];
  }
  __syncthreads();
  float2 *o = reinterpret_cast<float2 *>(out);
  for (int rl = w; rl < ry; rl += nw) {
    const int64_t row = row0 + rl;
    if (row >= rows) break;
    for (int k = lane; k < tn; k += 32) o[S.vox + row * W + x0 + k] = stage[rl * sstride + k];
  }
}

// ---------------------------------------------------------------- streaming y / x passes
// Radius-specialised min/max passes (L = 2R+1 known at compile time).  Each thread walks
// one line in blocks of L inputs and keeps, in registers, the suffix minima of the
// previous block and the running prefix minimum of the current one (van Herk /
// Gil-Werman): the window [t-R, t+R] starting at index i of block b is
// min(suffix_b[i], prefix_{b+1}[i-1]).  The loops over a block are unrolled, so every
// register index is a constant.  Nearest border (BORDER 0) clamps the line index; the
// zero border (BORDER 1) reads the packed zero outside the line.

// y pass: one thread per (column, segment of rows) of a slice; a warp reads 32
// consecutive columns of a row per load.
template <int R, int BORDER>
__global__ void __launch_bounds__(128, 8) k_mm_y_stream(const Sub *subs, int seg, const uint32_t *in, uint32_t *out) {
  constexpr int L = 2 * R + 1;
  const Sub S = subs[blockIdx.z];
  const int W = S.W, H = S.H;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int nseg = (H + seg - 1) / seg;
  const int z = blockIdx.y / nseg, ys = (blockIdx.y % nseg) * seg;
  if (x >= W || z >= S.D) return;
  const int ye = min(ys + seg, H);
  const int64_t plane = (int64_t)W * H;
  const uint32_t *col = in + S.vox + z * plane + x;
  uint32_t *oc = out + S.vox + z * plane + x;
  auto ld = [&](int y) -> uint32_t {
    if (BORDER == 1 && (y < 0 || y >= H)) return kZeroPacked;
    return __ldg(col + (int64_t)clampi(y, 0, H - 1) * W);
  };
  uint32_t suf[L], cur[L];
#pragma unroll
  for (int j = 0; j < L; j++) suf[j] = ld(ys - R + j);
#pragma unroll
  for (int j = L - 2; j >= 0; j--) suf[j] = __vminu2(suf[j], suf[j + 1]);
  for (int t0 = ys; t0 < ye; t0 += L) {
#pragma unroll
    for (int j = 0; j < L; j++) cur[j] = ld(t0 - R + L + j);
    uint32_t pre = 0xFFFFFFFFu;
#pragma unroll
    for (int i = 0; i < L; i++) {
      const uint32_t m = i == 0 ? suf[0] : __vminu2(suf[i], pre);
      if (t0 + i < ye) oc[(int64_t)(t0 + i) * W] = m;
      pre = __vminu2(pre, cur[i]);
    }
    suf[L - 1] = cur[L - 1];
#pragma unroll
    for (int j = L - 2; j >= 0; j--) suf[j] = __vminu2(cur[j], suf[j + 1]);
  }
}

// x pass (nearest border) with the exact x box sum -> float2 (ero_x, dil_x): one warp per
// 32 rows, one row per lane.  Each block of L inputs of the warp's rows is staged in
// shared memory by cp.async, one block ahead of the one in use (two buffers), then read
// one row per lane (L is odd, so the lanes' rows fall in distinct banks).  The box sum
// over the window minima M slides one position per step as an exact integer sum; the box
// output of u is formed when M(u + R) is, with M(0) standing for positions left of the
// row and M(W-1) right of it.  Outputs return through a shared tile for row-wise
// coalesced stores.
constexpr int kXsWarps = 2;

__device__ __forceinline__ void cp_async4(uint32_t *dst, const uint32_t *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <int R>
__global__ void __launch_bounds__(32 * kXsWarps) k_mm_x_stream(const Sub *subs, const uint32_t *in, float2 *out) {
  constexpr int L = 2 * R + 1;
  static_assert(L <= 255, "the integer box sum needs 2R+1 <= 256");
  __shared__ uint32_t sin_[kXsWarps][2][32 * L];
  __shared__ float2 sout[kXsWarps][32 * L];
  const Sub S = subs[blockIdx.y];
  const int W = S.W;
  const int64_t rows = (int64_t)S.H * S.D;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t row0 = ((int64_t)blockIdx.x * kXsWarps + w) * 32;
  if (row0 >= rows) return;
  const int nr = (int)min((int64_t)32, rows - row0);
  float2 *tout = sout[w];
  const uint32_t *lines = in + S.vox + row0 * W;
  float2 *olines = out + S.vox + row0 * W;

  // inputs [p, p + L) of the warp's rows (clamped to the row) -> buffer, asynchronously
  auto issue = [&](int p, uint32_t *buf) {
#pragma unroll 4
    for (int k = 0; k < 32; k++) {
      const uint32_t *line = lines + (int64_t)min(k, nr - 1) * W;
#pragma unroll
      for (int i = lane; i < L; i += 32) cp_async4(buf + k * L + i, line + clampi(p + i, 0, W - 1));
    }
    cp_async_commit();
  };

  const float inv = 1.0f / (float)L;
  const uint32_t full = (uint32_t)L * 0xFFFFu;
  uint32_t suf[L], cur[L], mp[L];
  issue(-R, sin_[w][0]);
  issue(-R + L, sin_[w][1]);
  cp_async_wait<1>();
  __syncwarp();
#pragma unroll
  for (int j = 0; j < L; j++) suf[j] = sin_[w][0][lane * L + j];
#pragma unroll
  for (int j = L - 2; j >= 0; j--) suf[j] = __vminu2(suf[j], suf[j + 1]);
  uint32_t slo = 0, shi = 0, m0 = 0, mlast = 0;
  int b = 0;
  for (int t0 = 0; t0 < W + R; t0 += L, b ^= 1) {
    __syncwarp();                                  // every lane is done with buffer b
    issue(t0 - R + 2 * L, sin_[w][b]);            // block after next
    cp_async_wait<1>();                            // block after this one has landed
    __syncwarp();
    const uint32_t *cb = sin_[w][b ^ 1];
#pragma unroll
    for (int j = 0; j < L; j++) cur[j] = cb[lane * L + j];
    uint32_t pre = 0xFFFFFFFFu;
    if (t0 >= L && t0 + L < W) {   // interior: every M(t - L) is in mp, no border
#pragma unroll
      for (int i = 0; i < L; i++) {
        const uint32_t m = i == 0 ? suf[0] : __vminu2(suf[i], pre);
        pre = __vminu2(pre, cur[i]);
        const uint32_t o = mp[i];
        slo += (m & 0xFFFFu) - (o & 0xFFFFu);
        shi += (m >> 16) - (o >> 16);
        mp[i] = m;
        tout[lane * L + i] = make_float2((float)slo * inv, (float)(full - shi) * inv);
      }
    } else {
#pragma unroll
      for (int i = 0; i < L; i++) {
        const int t = t0 + i;
        uint32_t m = i == 0 ? suf[0] : __vminu2(suf[i], pre);
        pre = __vminu2(pre, cur[i]);
        if (t == W - 1) mlast = m;
        if (t >= W) m = mlast;
        if (t == 0) {
          m0 = m;
          slo = (uint32_t)L * (m & 0xFFFFu);
          shi = (uint32_t)L * (m >> 16);
        } else {
          const uint32_t o = t >= L ? mp[i] : m0;
          slo += (m & 0xFFFFu) - (o & 0xFFFFu);
          shi += (m >> 16) - (o >> 16);
        }
        mp[i] = m;
        tout[lane * L + i] = make_float2((float)slo * inv, (float)(full - shi) * inv);
      }
    }
    __syncwarp();
    const int u0 = t0 - R;
#pragma unroll 4
    for (int k = 0; k < 32; k++) {
      if (k >= nr) break;
#pragma unroll
      for (int i = lane; i < L; i += 32) {
        const int u = u0 + i;
        if (u >= 0 && u < W) olines[(int64_t)k * W + u] = tout[k * L + i];
      }
    }
    __syncwarp();                                  // the tile is rewritten next block
    suf[L - 1] = cur[L - 1];
#pragma unroll
    for (int j = L - 2; j >= 0; j--) suf[j] = __vminu2(cur[j], suf[j + 1]);
  }
  cp_async_wait<0>();                              // no copy outlives the block
}

// ---------------------------------------------------------------- x pass (box, float chain)
// The literal float chain of the x box for windows wider than 256 (where the partial
// sums stop being exact integers), over a packed min/max volume.
__global__ void k_box_x_chain(const Sub *subs, int r, const uint32_t *in, float2 *out) {
  extern __shared__ float2 sfx[];
  constexpr int kSeg = 256;
  const Sub S = subs[blockIdx.y];
  const int segs = (S.W + kSeg - 1) / kSeg;
  const int64_t rows = (int64_t)S.H * S.D;
  const int64_t bid = blockIdx.x;
  if (bid >= rows * segs) return;
  const int64_t row = bid / segs;
  const int x0 = (int)(bid % segs) * kSeg;
  const int L = 2 * r + 1, n0 = kSeg + 2 * r;
  const float inv = 1.0f / (float)L;
  const uint32_t *line = in + S.vox + row * S.W;
  for (int i = threadIdx.x; i < n0; i += blockDim.x) {
    const uint32_t v = line[clampi(x0 - r + i, 0, S.W - 1)];
    sfx[i] = make_float2((float)mm_lo(v), (float)mm_hi(v));
  }
  __syncthreads();
  const int x = x0 + threadIdx.x;
  if (x >= S.W) return;
  float2 acc = make_float2(0.f, 0.f);
  for (int j = 0; j < L; j++) acc = add2(acc, sfx[threadIdx.x + j]);
  out[S.vox + row * S.W + x] = mul2(acc, make_float2(inv, inv));
}

// ---------------------------------------------------------------- y / z passes (box mean)
// Register-blocked sequential sums: a thread produces K consecutive outputs along the
// axis; slot (u + k) % K of a K-entry rotating window feeds output k at tap u of each
// block of K taps, so the window never moves between registers.  Every output still
// sums its 2r+1 inputs from 0.0f in the reference order.  load(i) returns input
// c0 - r + i.
template <int K, class LoadF>
__device__ __forceinline__ void box_chain(int L, LoadF load, float2 (&acc)[K]) {
  float2 win[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    win[k] = load(k);
    acc[k] = make_float2(0.f, 0.f);
  }
  int jb = 0;
  for (; jb + K <= L; jb += K) {
#pragma unroll
    for (int u = 0; u < K; u++) {
#pragma unroll
      for (int k = 0; k < K; k++) acc[k] = add2(acc[k], win[(u + k) % K]);
      win[u] = load(jb + u + K);
    }
  }
#pragma unroll
  for (int u = 0; u < K; u++) {
    if (jb + u < L) {
#pragma unroll
      for (int k = 0; k < K; k++) acc[k] = add2(acc[k], win[(u + k) % K]);
      if (jb + u + K < L + K - 1) win[u] = load(jb + u + K);
    }
  }
}

// The y box chain with a compile-time window: K outputs from a window of K registers
// (input j + k feeds output k at step j, in the reference's order: 0 + s0 + s1 + ...).
template <int K, int L, class LoadF>
__device__ __forceinline__ void box_chain_t(LoadF load, float2 (&acc)[K]) {
  float2 win[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    win[k] = load(k);
    acc[k] = make_float2(0.f, 0.f);
  }
#pragma unroll
  for (int j = 0; j < L; j++) {
#pragma unroll
    for (int k = 0; k < K; k++) acc[k] = add2(acc[k], win[(j + k) % K]);
    if (j + K < L + K - 1) win[j % K] = load(j + K);
  }
}

constexpr int kBoxYK = 12;   // y outputs per thread

__global__ void __launch_bounds__(128) k_box_y(const Sub *subs, int r, const float2 *in, float2 *out) {
  const Sub S = subs[blockIdx.y];
  const int rows_per_blk = blockDim.y * kBoxYK;
  const int tx_n = (S.W + 31) / 32, ty_n = (S.H + rows_per_blk - 1) / rows_per_blk;
  const int64_t bid = blockIdx.x;
  if (bid >= (int64_t)tx_n * ty_n * S.D) return;
  const int z = (int)(bid / ((int64_t)tx_n * ty_n));
  const int rem = (int)(bid % ((int64_t)tx_n * ty_n));
  const int x = (rem % tx_n) * 32 + threadIdx.x;
  const int y0 = (rem / tx_n) * rows_per_blk + threadIdx.y * kBoxYK;
  if (x >= S.W || y0 >= S.H) return;
  const int H = S.H, W = S.W, L = 2 * r + 1;
  const float2 *col = in + S.vox + (int64_t)z * W * H + x;
  float2 acc[kBoxYK];
  if (y0 - r >= 0 && y0 + kBoxYK + r <= H) {
    const float2 *p = col + (int64_t)(y0 - r) * W;
    box_chain<kBoxYK>(L, [&](int i) { return __ldg(p + (int64_t)i * W); }, acc);
  } else {
    box_chain<kBoxYK>(L, [&](int i) { return __ldg(col + (int64_t)clampi(y0 - r + i, 0, H - 1) * W); }, acc);
  }
  const float inv = 1.0f / (float)L;
  float2 *o = out + S.vox + (int64_t)z * W * H + x;
#pragma unroll
  for (int k = 0; k < kBoxYK; k++)
    if (y0 + k < H) o[(int64_t)(y0 + k) * W] = mul2(acc[k], make_float2(inv, inv));
}

// The y box with a compile-time radius: K outputs of one column per thread from a register
// window (box_chain_t), loads and stores walking running pointers, so that no address
// arithmetic joins the f32x2 adds in the FMA pipe.
template <int R, int K>
__global__ void __launch_bounds__(128, 6) k_box_y_t(const Sub *subs, const float2 *in, float2 *out) {
  constexpr int L = 2 * R + 1;
  const Sub S = subs[blockIdx.y];
  const int rows_per_blk = blockDim.y * K;
  const int tx_n = (S.W + 31) / 32, ty_n = (S.H + rows_per_blk - 1) / rows_per_blk;
  const int64_t bid = blockIdx.x;
  if (bid >= (int64_t)tx_n * ty_n * S.D) return;
  const int z = (int)(bid / ((int64_t)tx_n * ty_n));
  const int rem = (int)(bid % ((int64_t)tx_n * ty_n));
  const int x = (rem % tx_n) * 32 + threadIdx.x;
  const int y0 = (rem / tx_n) * rows_per_blk + threadIdx.y * K;
  if (x >= S.W || y0 >= S.H) return;
  const int H = S.H, W = S.W;
  const float2 *col = in + S.vox + (int64_t)z * W * H + x;
  float2 acc[K];
  if (y0 - R >= 0 && y0 + K + R <= H) {
    const float2 *q = col + (int64_t)(y0 - R) * W;   // box_chain_t loads its inputs in order
    box_chain_t<K, L>([&](int) {
      const float2 v = __ldg(q);
      q += W;
      return v;
    }, acc);
  } else {
    box_chain_t<K, L>([&](int i) { return __ldg(col + (int64_t)clampi(y0 - R + i, 0, H - 1) * W); }, acc);
  }
  const float inv = 1.0f / (float)L;
  float2 *o = out + S.vox + (int64_t)z * W * H + (int64_t)y0 * W + x;
#pragma unroll
  for (int k = 0; k < K; k++, o += W)
    if (y0 + k < H) *o = mul2(acc[k], make_float2(inv, inv));
}

// z pass of the box mean fused with Normalize3DKernel (NormalizeFilter.cu:571-586).
constexpr int kBoxZK = 8;

__global__ void __launch_bounds__(128) k_box_z_norm(const Sub *subs, int rz, float min_intensity, const float2 *in,
                                                    float *norm, float *ero_l, float *dil_l) {
  const Sub S = subs[blockIdx.y];
  const int64_t plane = (int64_t)S.W * S.H;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= plane) return;
  const float2 *col = in + S.vox + p;
  const int D = S.D, L = 2 * rz + 1;
  const float inv = 1.0f / (float)L;
  for (int z0 = 0; z0 < D; z0 += kBoxZK) {
    float2 acc[kBoxZK];
    box_chain<kBoxZK>(L, [&](int i) { return __ldg(col + clampi(z0 - rz + i, 0, D - 1) * plane); }, acc);
#pragma unroll
    for (int k = 0; k < kBoxZK; k++) {
      const int z = z0 + k;
      if (z < D) {
        const float2 el = mul2(acc[k], make_float2(inv, inv));
        const float v = z < S.depth_valid ? (float)__ldg(S.src + z * plane + p) : 0.0f;
        norm[S.vox + z * plane + p] = (v >= min_intensity) ? (v - el.x) / (el.y - el.x) : 0.0f;
        if (ero_l) {
          ero_l[S.vox + z * plane + p] = el.x;
          dil_l[S.vox + z * plane + p] = el.y;
        }
      }
    }
  }
}

// The same pass specialised on the z radius: one thread per (column, chunk of kBoxZK
// slices), every window input loaded before the first add so that all loads of a thread
// are in flight together; threadIdx.y picks the chunk, so the chunks of one column share
// their overlapping inputs through L1.  PARTS also stores the box means (stage dumps).
template <int RZ, bool PARTS>
__global__ void __launch_bounds__(128) k_box_z_norm_t(const Sub *subs, float min_intensity, const float2 *in,
                                                      float *norm, float *ero_l, float *dil_l) {
  constexpr int L = 2 * RZ + 1, NW = kBoxZK + 2 * RZ;
  const Sub S = subs[blockIdx.z];
  const int64_t plane = (int64_t)S.W * S.H;
  const int64_t p = (int64_t)blockIdx.x * 32 + threadIdx.x;
  const int z0 = (blockIdx.y * blockDim.y + threadIdx.y) * kBoxZK;
  const int D = S.D;
  if (p >= plane || z0 >= D) return;
  const float2 *col = in + S.vox + p;
  float2 win[NW];
#pragma unroll
  for (int i = 0; i < NW; i++) win[i] = __ldg(col + clampi(z0 - RZ + i, 0, D - 1) * plane);
  float v[kBoxZK];
#pragma unroll
  for (int k = 0; k < kBoxZK; k++) {
    const int z = min(z0 + k, D - 1);
    v[k] = z < S.depth_valid ? (float)__ldg(S.src + z * plane + p) : 0.0f;
  }
  const float inv = 1.0f / (float)L;
#pragma unroll
  for (int k = 0; k < kBoxZK; k++) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < L; j++) acc = add2(acc, win[k + j]);
    const int z = z0 + k;
    if (z < D) {
      const float2 el = mul2(acc, make_float2(inv, inv));
      norm[S.vox + z * plane + p] = (v[k] >= min_intensity) ? (v[k] - el.x) / (el.y - el.x) : 0.0f;
      if (PARTS) {
        ero_l[S.vox + z * plane + p] = el.x;
        dil_l[S.vox + z * plane + p] = el.y;
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

// ---------------------------------------------------------------- launchers
static int max_optin_smem() {
  static int v = 0;
  if (!v) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (v <= 0) v = 48 * 1024;
  }
  return v;
}

template <class F>
static void allow_smem(F *fn, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int BORDER>
static void mm_z(const Sub *d_subs, int nsub, int plane, int rz, bool vec4, uint32_t *mm, cudaStream_t s) {
  if (BORDER == 0 && vec4 && rz == 5) {
    dim3 grid(ceil_div(plane / 2, 128), nsub);
    KLAUNCH("k_mm_z", s, (k_mm_z_stream<5><<<grid, 128, 0, s>>>(d_subs, mm)));
  } else if (vec4) {
    dim3 grid(ceil_div(plane / 4, 256), nsub);
    KLAUNCH("k_mm_z", s, (k_mm_z<BORDER, 4><<<grid, 256, 0, s>>>(d_subs, rz, mm)));
  } else {
    dim3 grid(ceil_div(plane, 256), nsub);
    KLAUNCH("k_mm_z", s, (k_mm_z<BORDER, 1><<<grid, 256, 0, s>>>(d_subs, rz, mm)));
  }
}

template <int BORDER>
static void mm_y(const Sub *d_subs, int nsub, int W, int H, int D, int r, const uint32_t *in, uint32_t *out,
                 cudaStream_t s) {
  // rows per block: 128, fewer when the staged window would not fit in shared memory
  const int cap_rows = max_optin_smem() / (2 * 32 * 4);
  int ty = 128;
  while (ty > 16 && ty + 2 * r > cap_rows) ty /= 2;
  const size_t smem = (size_t)2 * (ty + 2 * r) * 32 * 4;
  allow_smem(k_mm_y<BORDER>, smem);
  dim3 grid((unsigned)((int64_t)ceil_div(W, 32) * ceil_div(H, ty) * D), nsub);
  KLAUNCH("k_mm_y", s, (k_mm_y<BORDER><<<grid, 256, smem, s>>>(d_subs, r, ty, in, out)));
}

// The streaming passes where the radius has an instantiation (false: use the staged ones).
template <int BORDER>
static bool mm_y_stream(const Sub *d_subs, int nsub, int W, int H, int D, int r, const uint32_t *in, uint32_t *out,
                        cudaStream_t s) {
  const int L = 2 * r + 1;
  const int seg = (ceil_div(H, 4) + L - 1) / L * L;   // about four segments a column, whole blocks
  const dim3 grid(ceil_div(W, 128), ceil_div(H, seg) * D, nsub);
  switch (r) {
    case 20:
      KLAUNCH("k_mm_y", s, (k_mm_y_stream<20, BORDER><<<grid, 128, 0, s>>>(d_subs, seg, in, out)));
      return true;
    default:
      return false;
  }
}

static bool mm_x_stream(const Sub *d_subs, int nsub, int64_t rows, int r, const uint32_t *in, float2 *out,
                        cudaStream_t s) {
  const dim3 grid(ceil_div(rows, 32 * kXsWarps), nsub);
  switch (r) {
    case 20:
      KLAUNCH("k_mm_x", s, (k_mm_x_stream<20><<<grid, 32 * kXsWarps, 0, s>>>(d_subs, in, out)));
      return true;
    default:
      return false;
  }
}

static size_t mm_x_smem(int mode, int r, int ry, int tx) {
  const int hm = mode == 0 ? r : 0;
  const int stride = (tx + 2 * hm + 2 * r) | 1;
  size_t words = (size_t)2 * ry * stride;
  if (mode == 0) {
    words += (size_t)ry * ((tx + 2 * r) | 1);
    words = words > (size_t)ry * (tx + 1) * 2 ? words : (size_t)ry * (tx + 1) * 2;   // staging fits over A + G
  }
  return words * 4;
}

template <int BORDER, int MODE>
static void mm_x(const Sub *d_subs, int nsub, int W, int64_t rows, int r, const uint32_t *in, void *out,
                 cudaStream_t s) {
  // 16 rows x 256 outputs per block, narrower until the staged rows fit in shared
  // memory; MODE 0 runs one thread per (row, chunk of kBoxC outputs).
  int ry = 16, tx = 256;
  while (mm_x_smem(MODE, r, ry, tx) > (size_t)max_optin_smem() && tx > 64) tx /= 2;
  const size_t smem = mm_x_smem(MODE, r, ry, tx);
  const int threads = MODE == 0 ? ry * (tx / kBoxC) : 256;
  allow_smem(k_mm_x<BORDER, MODE>, smem);
  dim3 grid((unsigned)(((rows + ry - 1) / ry) * ceil_div(W, tx)), nsub);
  KLAUNCH("k_mm_x", s, (k_mm_x<BORDER, MODE><<<grid, threads, smem, s>>>(d_subs, r, ry, tx, in, out)));
}

void launch_normalize(const Sub *d_subs, int nsub, int W, int H, int D, int rxy, int rz, float min_intensity,
                      bool src_aligned8, uint32_t *ma, uint32_t *mb, float2 *fa, float2 *fb, float *norm,
                      cudaStream_t s, float *ero_l, float *dil_l) {
  const int plane = W * H;
  const int64_t rows = (int64_t)H * D;
  mm_z<0>(d_subs, nsub, plane, rz, src_aligned8 && plane % 4 == 0, ma, s);
  if (!mm_y_stream<0>(d_subs, nsub, W, H, D, rxy, ma, mb, s)) mm_y<0>(d_subs, nsub, W, H, D, rxy, ma, mb, s);
  if (mm_x_stream(d_subs, nsub, rows, rxy, mb, fa, s)) {
  } else if (2 * rxy + 1 <= 256) {
    mm_x<0, 0>(d_subs, nsub, W, rows, rxy, mb, fa, s);
  } else {
    mm_x<0, 2>(d_subs, nsub, W, rows, rxy, mb, ma, s);
    const size_t smem = (size_t)(256 + 2 * rxy) * sizeof(float2);
    allow_smem(k_box_x_chain, smem);
    KLAUNCH("k_box_x_chain", s, (k_box_x_chain<<<dim3((unsigned)(rows * ceil_div(W, 256)), nsub), 256, smem, s>>>(
                                    d_subs, rxy, ma, fa)));
  }
  const int by = 4;
  if (rxy == 20) {   // the workload's radius: compile-time window, 16 outputs a thread
    constexpr int K = 16;
    dim3 gy((unsigned)((int64_t)ceil_div(W, 32) * ceil_div(H, by * K) * D), nsub);
    KLAUNCH("k_box_y", s, (k_box_y_t<20, K><<<gy, dim3(32, by), 0, s>>>(d_subs, fa, fb)));
  } else {
    dim3 gy((unsigned)((int64_t)ceil_div(W, 32) * ceil_div(H, by * kBoxYK) * D), nsub);
    KLAUNCH("k_box_y", s, (k_box_y<<<gy, dim3(32, by), 0, s>>>(d_subs, rxy, fa, fb)));
  }
  const dim3 gz(ceil_div(plane, 32), ceil_div(D, 4 * kBoxZK), nsub), bz(32, 4);
  switch (rz) {
#define HDOG_BOXZ_CASE(R)                                                                                   \
  case R:                                                                                                   \
    if (ero_l)                                                                                              \
      KLAUNCH("k_box_z_norm", s, (k_box_z_norm_t<R, true><<<gz, bz, 0, s>>>(d_subs, min_intensity, fb, norm, ero_l, dil_l))); \
    else                                                                                                    \
      KLAUNCH("k_box_z_norm", s, (k_box_z_norm_t<R, false><<<gz, bz, 0, s>>>(d_subs, min_intensity, fb, norm, ero_l, dil_l))); \
    break;
    HDOG_BOXZ_CASE(1) HDOG_BOXZ_CASE(2) HDOG_BOXZ_CASE(3) HDOG_BOXZ_CASE(4)
    HDOG_BOXZ_CASE(5) HDOG_BOXZ_CASE(6) HDOG_BOXZ_CASE(7) HDOG_BOXZ_CASE(8)
#undef HDOG_BOXZ_CASE
    default:
      KLAUNCH("k_box_z_norm", s, (k_box_z_norm<<<dim3(ceil_div(plane, 128), nsub), 128, 0, s>>>(
                                     d_subs, rz, min_intensity, fb, norm, ero_l, dil_l)));
  }
}

void launch_copy_norm(const Sub *d_subs, int nsub, int64_t max_n, float min_intensity, float *norm,
                      cudaStream_t s) {
  dim3 grid(ceil_div(max_n, 256), nsub);
  KLAUNCH("k_copy_norm", s, (k_copy_norm<<<grid, 256, 0, s>>>(d_subs, min_intensity, norm)));
}

// Erosion3DFilter: min with a zero border.  Min is separable and exact, so z -> y -> x
// gives the reference's x -> y -> z result.  `tmp` holds two packed u32 volumes.
void launch_erosion(const Sub *d_subs, int nsub, int W, int H, int D, int rxy, int rz, bool src_aligned8,
                    uint32_t *tmp, uint16_t *dst, cudaStream_t s) {
  const int plane = W * H;
  const int64_t n = (int64_t)plane * D;
  uint32_t *a = tmp, *b = tmp + n * nsub;
  mm_z<1>(d_subs, nsub, plane, rz, src_aligned8 && plane % 4 == 0, a, s);
  mm_y<1>(d_subs, nsub, W, H, D, rxy, a, b, s);
  mm_x<1, 1>(d_subs, nsub, W, (int64_t)H * D, rxy, b, dst, s);
}

}  // namespace hdog
