// regions.cu -- region numbering, per-region features, eigen features and candidate
// records, sm_103a.
//
// Reference: src/3D/RegionalFeatures.cu (HessianFeatures :295-329, MaxNormalized :65-87,
// SumNormalized :114-137, RegionalSizeAndCentroid :214-255), src/3D/Eigenvalues.cu
// (:19-112) and src/3D/utils.h (saveFeatureVector :204-250).
//
// The reference runs ten full-volume radix sorts (label -> value) and reduce-by-key.
// Here regions are numbered by a scan over the root bitmap the labelling pass leaves
// (ascending root index = the reference's region order), and one pass over the
// foreground accumulates count, max intensity, exact integer coordinate sums and the
// six Hessian sums (recomputed from the DoG instead of stored) with integer atomics:
// fixed point for the float sums, so the result does not depend on thread order.
#include "kernels.cuh"

namespace hdog {

// ------------------------------------------------------------------ segmented scan
// Exclusive scan of per-block counts, independently per substack.  seg_off/seg_len
// locate each substack's count array; chunk scratch holds one sum per 1024 counts.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t wsum[33];   // [0, 32): exclusive warp offsets, [32]: block total
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t s = lane < nw ? wsum[lane] : 0u, si = s;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, si, o);
      if (lane >= o) si += y;
    }
    if (lane < nw) wsum[lane] = si - s;
    if (lane == nw - 1) wsum[32] = si;
  }
  __syncthreads();
  const uint32_t r = wsum[w] + inc - v;
  if (total) *total = wsum[32];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(1024) k_scan_p1(const int64_t *seg_off, const int64_t *seg_len,
                                                  const int64_t *chk_off, const uint32_t *in,
                                                  uint32_t *chunk) {
  const int s = blockIdx.y;
  const int64_t len = seg_len[s], c = blockIdx.x;
  if (c * 1024 >= len) return;
  const int64_t i = c * 1024 + threadIdx.x;
  uint32_t v = i < len ? in[seg_off[s] + i] : 0u;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  __shared__ uint32_t ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t t = ws[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xFFFFFFFFu, t, o);
    if (threadIdx.x == 0) chunk[chk_off[s] + c] = t;
  }
}

// One block per substack: exclusive scan of its chunk sums; total -> totals[s].
__global__ void __launch_bounds__(1024) k_scan_p2(const int64_t *seg_len, const int64_t *chk_off,
                                                  uint32_t *chunk, int64_t *totals, int64_t add) {
  const int s = blockIdx.x;
  const int64_t nch = (seg_len[s] + 1023) / 1024;
  uint32_t carry = 0;
  for (int64_t b = 0; b < nch; b += 1024) {
    const int64_t i = b + threadIdx.x;
    const uint32_t v = i < nch ? chunk[chk_off[s] + i] : 0u;
    uint32_t tot;
    const uint32_t e = block_excl_scan(v, &tot);
    if (i < nch) chunk[chk_off[s] + i] = carry + e;
    carry += tot;
  }
  if (threadIdx.x == 0) totals[s] = (int64_t)carry + add;
}

__global__ void __launch_bounds__(1024) k_scan_p3(const int64_t *seg_off, const int64_t *seg_len,
                                                  const int64_t *chk_off, const uint32_t *in,
                                                  const uint32_t *chunk, uint32_t *out) {
  const int s = blockIdx.y;
  const int64_t len = seg_len[s], c = blockIdx.x;
  if (c * 1024 >= len) return;
  const int64_t i = c * 1024 + threadIdx.x;
  const uint32_t v = i < len ? in[seg_off[s] + i] : 0u;
  const uint32_t e = block_excl_scan(v, nullptr);
  if (i < len) out[seg_off[s] + i] = chunk[chk_off[s] + c] + e;
}

// ------------------------------------------------------------------ region numbering
// Region r >= 1 is the r-th root in ascending voxel order (region 0 = background), the
// order reduce-by-key over sorted labels produces.  Each root initialises its slot.
__device__ __forceinline__ void init_slot(RegionAcc acc, int64_t slots, int64_t g, int32_t label) {
  acc.label[g] = label;
  acc.count[g] = 0u;
  acc.max_ord[g] = 0u;   // below f2ord of every float
  acc.sum_norm[g] = 0ull;
#pragma unroll
  for (int k = 0; k < 3; k++) acc.sum_xyz[k * slots + g] = 0ull;
#pragma unroll
  for (int k = 0; k < 6; k++) acc.hess[k * slots + g] = 0ull;
}

// 4096 voxels per block, 16 per thread; the thread's root bits are one half-word.
// One block of kRankThreads threads per kScanBlock voxels, 64 voxels (two root-bit words)
// per thread: roots numbered in voxel order after the block's offset.
constexpr int kRankThreads = kScanBlock / 64;

__global__ void __launch_bounds__(kRankThreads) k_rank(const Sub *subs, const uint32_t *root_bits,
                                                       const uint32_t *blk_offsets, int32_t *rank, RegionAcc acc,
                                                       int64_t slots, int *status) {
  const Sub S = subs[blockIdx.y];
  const int64_t n = (int64_t)S.W * S.H * S.D;
  const int64_t base = (int64_t)blockIdx.x * kScanBlock;
  if (base >= n) return;
  const uint2 w = reinterpret_cast<const uint2 *>(root_bits + (S.blk + blockIdx.x) * (kScanBlock / 32))[threadIdx.x];
  const uint32_t pre = block_excl_scan(__popc(w.x) + __popc(w.y), nullptr);
  if (blockIdx.x == 0 && threadIdx.x == 0) init_slot(acc, slots, S.reg, 0);
  int64_t r = 1 + (int64_t)blk_offsets[S.blk + blockIdx.x] + pre;
  for (int half = 0; half < 2; half++) {
    uint32_t bits = half ? w.y : w.x;
    while (bits) {
      const int k = __ffs(bits) - 1;
      bits &= bits - 1;
      if (r >= S.reg_cap) { atomicExch(status, HDOG_ERR_CAPACITY); return; }
      const int64_t i = base + threadIdx.x * 64 + half * 32 + k;
      rank[S.vox + i] = (int32_t)r;
      init_slot(acc, slots, S.reg + r, (int32_t)i);
      r++;
    }
  }
}

// Per-run partial sums of one thread: consecutive foreground voxels of one region are
// summed in registers and flushed with one atomic per field.  All sums are integers
// (fixed point for the float ones), so the result is independent of the flush order.
struct RunAcc {
  int64_t r;
  uint32_t count, max_ord;
  unsigned long long norm, x, y, z, h[6];
};

__device__ __forceinline__ void run_reset(RunAcc &a, int64_t r) {
  a.r = r; a.count = 0; a.max_ord = 0; a.norm = a.x = a.y = a.z = 0ull;
#pragma unroll
  for (int k = 0; k < 6; k++) a.h[k] = 0ull;
}

__device__ __forceinline__ void run_flush(const RunAcc &a, const Sub &S, RegionAcc acc, int64_t slots) {
  if (a.r <= 0 || a.r >= S.reg_cap || a.count == 0) return;
  const int64_t g = S.reg + a.r;
  atomicAdd(&acc.count[g], a.count);
  atomicMax(&acc.max_ord[g], a.max_ord);
  atomicAdd(&acc.sum_norm[g], a.norm);
  atomicAdd(&acc.sum_xyz[g], a.x);
  atomicAdd(&acc.sum_xyz[slots + g], a.y);
  atomicAdd(&acc.sum_xyz[2 * slots + g], a.z);
#pragma unroll
  for (int k = 0; k < 6; k++) atomicAdd(&acc.hess[k * slots + g], a.h[k]);
}

// One pass over the foreground: count, max / sum of normalized intensity, exact
// coordinate sums, Hessian element sums.  mask may be null: foreground = label != 0.
__global__ void __launch_bounds__(256) k_accumulate(const Sub *subs, const uint8_t *mask, const int32_t *labels,
                                                    const int32_t *rank, const float *norm, const float *dog,
                                                    RegionAcc acc, int64_t slots) {
  const Sub S = subs[blockIdx.y];
  const int64_t n = (int64_t)S.W * S.H * S.D;
  const int64_t i0 = (int64_t)blockIdx.x * kScanBlock + threadIdx.x * 16;
  if (i0 >= n) return;
  uint8_t mk[16];
  if (mask) {
    const uint8_t *m = mask + S.vox;
    if (i0 + 16 <= n && ((reinterpret_cast<uintptr_t>(m + i0) & 15) == 0)) {
      *reinterpret_cast<uint4 *>(mk) = __ldg(reinterpret_cast<const uint4 *>(m + i0));
    } else {
      for (int k = 0; k < 16; k++) mk[k] = (i0 + k < n) ? m[i0 + k] : 0;
    }
  } else {
    for (int k = 0; k < 16; k++) mk[k] = (i0 + k < n) ? (labels[S.vox + i0 + k] != 0) : 0;
  }
  RunAcc a;
  run_reset(a, -1);
  const int W = S.W, H = S.H;
  for (int k = 0; k < 16; k++) {
    const int64_t i = i0 + k;
    if (i == 0 || !mk[k]) continue;
    const int32_t lab = labels[S.vox + i];
    const int64_t r = rank[S.vox + lab];
    if (r != a.r) {
      run_flush(a, S, acc, slots);
      run_reset(a, r);
    }
    const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)(i / ((int64_t)W * H));
    const float v = norm[S.vox + i];
    a.count++;
    a.max_ord = max(a.max_ord, f2ord(v));
    a.norm += to_fix(v);
    a.x += (unsigned long long)x;
    a.y += (unsigned long long)y;
    a.z += (unsigned long long)z;
    float h[6];
    hessian_at(dog + S.vox, W, H, S.D, x, y, z, h);
#pragma unroll
    for (int q = 0; q < 6; q++) a.h[q] += to_fix(h[q]);
  }
  run_flush(a, S, acc, slots);
}

// The same accumulation from the foreground list of the fused sweep, a warp at a time:
// lane l takes entry e0 + 32 j + l (coalesced), consecutive entries of one region (the
// sweep appends the foreground of a 32 x 4 patch at a time, so runs are long) are summed
// across the warp by a segmented shuffle scan, and only the last lane of each run issues
// the atomics.  A run that reaches lane 31 carries into lane 0 of the next 32 entries, so
// a region's sums leave the warp once per kAccSpan-entry task at most.  All sums are
// integers (fixed point for the float ones), so the grouping does not change them.
constexpr int kAccSpan = 512;   // entries per warp task
static_assert((long long)kAccSpan * 65535 < (1ll << 32), "32-bit coordinate sums of a warp task");

// Sums of one run inside a warp task: the coordinate sums of at most kAccSpan entries fit
// 32 bits because the list path runs only for frames below 2^16 voxels on every axis
// (they widen to 64 bits in the atomics).
struct RunSums {
  uint32_t count, max_ord, x, y, z;
  unsigned long long norm, h[6];
};

__device__ __forceinline__ void sums_add(RunSums &a, const RunSums &b) {
  a.count += b.count;
  a.max_ord = max(a.max_ord, b.max_ord);
  a.norm += b.norm;
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
#pragma unroll
  for (int k = 0; k < 6; k++) a.h[k] += b.h[k];
}

__device__ __forceinline__ RunSums sums_shfl_up(const RunSums &a, int d) {
  RunSums b;
  b.count = __shfl_up_sync(0xFFFFFFFFu, a.count, d);
  b.max_ord = __shfl_up_sync(0xFFFFFFFFu, a.max_ord, d);
  b.norm = __shfl_up_sync(0xFFFFFFFFu, a.norm, d);
  b.x = __shfl_up_sync(0xFFFFFFFFu, a.x, d);
  b.y = __shfl_up_sync(0xFFFFFFFFu, a.y, d);
  b.z = __shfl_up_sync(0xFFFFFFFFu, a.z, d);
#pragma unroll
  for (int k = 0; k < 6; k++) b.h[k] = __shfl_up_sync(0xFFFFFFFFu, a.h[k], d);
  return b;
}

__device__ __forceinline__ RunSums sums_shfl(const RunSums &a, int src) {
  RunSums b;
  b.count = __shfl_sync(0xFFFFFFFFu, a.count, src);
  b.max_ord = __shfl_sync(0xFFFFFFFFu, a.max_ord, src);
  b.norm = __shfl_sync(0xFFFFFFFFu, a.norm, src);
  b.x = __shfl_sync(0xFFFFFFFFu, a.x, src);
  b.y = __shfl_sync(0xFFFFFFFFu, a.y, src);
  b.z = __shfl_sync(0xFFFFFFFFu, a.z, src);
#pragma unroll
  for (int k = 0; k < 6; k++) b.h[k] = __shfl_sync(0xFFFFFFFFu, a.h[k], src);
  return b;
}

__device__ __forceinline__ void sums_flush(const RunSums &a, int64_t r, const Sub &S, RegionAcc acc, int64_t slots) {
  if (r <= 0 || r >= S.reg_cap || a.count == 0) return;
  const int64_t g = S.reg + r;
  atomicAdd(&acc.count[g], a.count);
  atomicMax(&acc.max_ord[g], a.max_ord);
  atomicAdd(&acc.sum_norm[g], a.norm);
  atomicAdd(&acc.sum_xyz[g], (unsigned long long)a.x);
  atomicAdd(&acc.sum_xyz[slots + g], (unsigned long long)a.y);
  atomicAdd(&acc.sum_xyz[2 * slots + g], (unsigned long long)a.z);
#pragma unroll
  for (int k = 0; k < 6; k++) atomicAdd(&acc.hess[k * slots + g], a.h[k]);
}

__global__ void __launch_bounds__(256) k_accumulate_fg(const Sub *subs, const FgEntry *fg,
                                                       const unsigned long long *fg_count, const int32_t *fg_root,
                                                       const int32_t *rank, RegionAcc acc, int64_t slots) {
  const Sub S = subs[blockIdx.y];
  const int64_t cnt = (int64_t)fg_count[blockIdx.y * kFgCountStride];
  if (cnt > S.fg_cap) return;   // overflowed: the batch is redone without the fused sweep
  const int W = S.W, H = S.H;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const float4 *ent = reinterpret_cast<const float4 *>(fg + S.fg);
  for (int64_t e0 = warp * kAccSpan; e0 < cnt; e0 += nwarps * kAccSpan) {
    const int64_t e1 = min(e0 + kAccSpan, cnt);
    RunSums carry = {};   // the run that reached lane 31 of the previous 32 entries (same in every lane)
    int32_t ck = -1;      // its region
    for (int64_t b = e0; b < e1; b += 32) {
      const int64_t e = b + lane;
      RunSums v = {};
      int32_t key = -1;
      if (e < e1) {
        const float4 q0 = __ldg(ent + 2 * e), q1 = __ldg(ent + 2 * e + 1);
        key = rank[S.vox + __ldg(fg_root + S.fg + e)];
        const int32_t i = __float_as_int(q0.x);
        v.count = 1;
        v.max_ord = f2ord(q0.y);
        v.norm = to_fix(q0.y);
        v.x = (uint32_t)(i % W);
        v.y = (uint32_t)((i / W) % H);
        v.z = (uint32_t)(i / (W * H));
        v.h[0] = to_fix(q0.z);
        v.h[1] = to_fix(q0.w);
        v.h[2] = to_fix(q1.x);
        v.h[3] = to_fix(q1.y);
        v.h[4] = to_fix(q1.z);
        v.h[5] = to_fix(q1.w);
      }
      // the carried run joins lane 0's run, or leaves the warp
      if (lane == 0) {
        if (key == ck) sums_add(v, carry);
        else sums_flush(carry, ck, S, acc, slots);
      }
      const int32_t prev = __shfl_up_sync(0xFFFFFFFFu, key, 1);
      const uint32_t heads = __ballot_sync(0xFFFFFFFFu, lane == 0 || key != prev);
      const int start = 31 - __clz(heads & (0xFFFFFFFFu >> (31 - lane)));   // first lane of this run
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const RunSums u = sums_shfl_up(v, d);
        if (lane - d >= start) sums_add(v, u);
      }
      // last lane of a run that ends inside these 32 entries: flush; lane 31 carries
      if (lane != 31 && ((heads >> (lane + 1)) & 1u)) sums_flush(v, key, S, acc, slots);
      carry = sums_shfl(v, 31);
      ck = __shfl_sync(0xFFFFFFFFu, key, 31);
    }
    if (lane == 0) sums_flush(carry, ck, S, acc, slots);
  }
}

// ------------------------------------------------------------------ eigen features
// EigenvaluesKernel<float> (Eigenvalues.cu:19-96): Eberly's closed form in double on
// the float region sums; structureness = l0^2 + l1^2 + l2^2, blobness = l2^2 / (l0*l1).
__device__ void eigen_features(const float hs[6], float *structureness, float *blobness) {
  const double xx = hs[0], xy = hs[1], xz = hs[2], yy = hs[3], yz = hs[4], zz = hs[5];
  const double max0 = fmax(fabs(xx), fabs(xy));
  const double max1 = fmax(fabs(xz), fabs(yy));
  const double max2 = fmax(fabs(yz), fabs(zz));
  const double maxAbs = fmax(fmax(max0, max1), max2);
  if (maxAbs < 1e-30) { *structureness = 0.f; *blobness = 0.f; return; }
  const double nrm = xy * xy + xz * xz + yz * yz;
  double e0, e1, e2;
  if (nrm > 1e-30) {
    const double t = (xx + yy + zz) / 3.0;
    const double b00 = xx - t, b11 = yy - t, b22 = zz - t;
    const double den = sqrt((b00 * b00 + b11 * b11 + b22 * b22 + nrm * 2.0) / 6.0);
    const double c00 = b11 * b22 - yz * yz;
    const double c01 = xy * b22 - yz * xz;
    const double c02 = xy * yz - b11 * xz;
    const double det = (b00 * c00 - xy * c01 + xz * c02) / (den * den * den);
    const double hd = fmin(fmax(det * 0.5, -1.0), 1.0);
    const double ang = acos(hd) / 3.0;
    const double twoThirdsPi = 2.094395102393195;
    const double beta2 = cos(ang) * 2.0;
    const double beta0 = cos(ang + twoThirdsPi) * 2.0;
    const double beta1 = -(beta0 + beta2);
    e0 = t + den * beta0;
    e1 = t + den * beta1;
    e2 = t + den * beta2;
  } else {
    e0 = xx; e1 = yy; e2 = zz;
  }
  *structureness = (float)(e0 * e0 + e1 * e1 + e2 * e2);
  *blobness = (float)(e2 * e2 / (e0 * e1));
}

// Per region: float features, eigen features and the saveFeatureVector filter
// (utils.h:222-232); keep counts per block of kFinalizeBlock regions.
__global__ void __launch_bounds__(kFinalizeBlock) k_finalize(const Sub *subs, const int64_t *num_regions,
                                                            RegionAcc acc, int64_t slots, RegionOut out,
                                                            FilterParams fp, uint32_t *blk_counts) {
  const Sub S = subs[blockIdx.y];
  const int64_t R = min(num_regions[blockIdx.y], S.reg_cap);
  __shared__ uint32_t wc[kFinalizeBlock / 32];
  // only the blocks that hold regions (the counts of the others were zeroed)
  for (int64_t blk = blockIdx.x; blk * kFinalizeBlock < R; blk += gridDim.x) {
  const int64_t r = blk * kFinalizeBlock + threadIdx.x;
  bool keep = false;
  if (r < R) {
    const int64_t g = S.reg + r;
    const uint32_t cnt = acc.count[g];
    const float c16 = (float)(uint16_t)(cnt & 0xFFFFu);
    const float cx = __fdiv_rn(__ull2float_rn(acc.sum_xyz[g]), c16);
    const float cy = __fdiv_rn(__ull2float_rn(acc.sum_xyz[slots + g]), c16);
    const float cz = __fdiv_rn(__ull2float_rn(acc.sum_xyz[2 * slots + g]), c16);
    const float inten = fp.is_ave_mode ? __double2float_rn(from_fix(acc.sum_norm[g])) : ord2f(acc.max_ord[g]);
    float hs[6];
#pragma unroll
    for (int k = 0; k < 6; k++) hs[k] = __double2float_rn(from_fix(acc.hess[k * slots + g]));
    out.intensity[g] = inten;
    out.centroid[g] = cx; out.centroid[slots + g] = cy; out.centroid[2 * slots + g] = cz;
#pragma unroll
    for (int k = 0; k < 6; k++) out.hessian[k * slots + g] = hs[k];
    if (r >= 1) {
      keep = true;
      if (cz < (float)S.margin || cz >= (float)(S.depth_valid - S.margin)) keep = false;
      if (cx < (float)fp.left || cx >= (float)(S.W - fp.right)) keep = false;
      if (cy < (float)fp.top || cy >= (float)(S.H - fp.bottom)) keep = false;
      if ((int)(cnt & 0xFFFFu) < fp.min_size || inten <= 0.0f) keep = false;
    }
    // the FP64 eigen solve only where its result is read
    if (keep || fp.all_eigen) {
      float st, bl;
      eigen_features(hs, &st, &bl);
      out.eigen[g] = st; out.eigen[slots + g] = bl;
    }
    out.keep[g] = keep ? 1 : 0;
  }
  const uint32_t b = __ballot_sync(0xFFFFFFFFu, keep);
  if ((threadIdx.x & 31) == 0) wc[threadIdx.x >> 5] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int k = 0; k < kFinalizeBlock / 32; k++) t += wc[k];
    blk_counts[S.blk + blk] = t;
  }
  __syncthreads();   // wc is rewritten by the next block
  }
}

// Write kept regions as 28-byte records in region order (FeatureVector, utils.h:235-246).
__global__ void __launch_bounds__(kFinalizeBlock) k_records(const Sub *subs, const int64_t *num_regions,
                                                           RegionOut out, const uint32_t *count,
                                                           int64_t slots, const uint32_t *blk_offsets,
                                                           hdog_record *rec) {
  const Sub S = subs[blockIdx.y];
  const int64_t R = min(num_regions[blockIdx.y], S.reg_cap);
  __shared__ uint32_t wp[kFinalizeBlock / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t blk = blockIdx.x; blk * kFinalizeBlock < R; blk += gridDim.x) {
  const int64_t r = blk * kFinalizeBlock + threadIdx.x;
  const int64_t g = S.reg + r;
  const bool keep = r < R && out.keep[g];
  const uint32_t b = __ballot_sync(0xFFFFFFFFu, keep);
  if (lane == 0) wp[w] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int k = 0; k < kFinalizeBlock / 32; k++) { const uint32_t c = wp[k]; wp[k] = t; t += c; }
  }
  __syncthreads();
  if (keep) {
  const int64_t o = S.reg + blk_offsets[S.blk + blk] + wp[w] + __popc(b & ((1u << lane) - 1u));
  hdog_record q;
  q.centroid_x = out.centroid[g];
  q.centroid_y = out.centroid[slots + g];
  q.centroid_z = __fadd_rn(out.centroid[2 * slots + g], (float)S.z0);
  q.structureness = out.eigen[g];
  q.blobness = out.eigen[slots + g];
  q.intensity = out.intensity[g];
  q.size = (uint16_t)(count[g] & 0xFFFFu);
  q.padding = 0;
  rec[o] = q;
  }
  __syncthreads();   // wp is rewritten by the next block
  }
}


// ------------------------------------------------------------------ zero fill
// Clearing by a kernel rather than cudaMemsetAsync: a memset can go to a copy engine, where
// it would queue behind the chunks of a host stack being copied on the copy stream.
__global__ void k_zero32(uint32_t *p, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = 0u;
}

void zero_async(void *p, size_t bytes, cudaStream_t s) {
  const int64_t n = (int64_t)(bytes / 4);
  if (n > 0)
    KLAUNCH("k_zero32", s, (k_zero32<<<(unsigned)std::min<int64_t>(ceil_div(n, 256), 4096), 256, 0, s>>>(
                               static_cast<uint32_t *>(p), n)));
}

// The substacks' list counters (kFgCountStride apart) into consecutive slots, for one
// plain device-to-host copy.
__global__ void k_pack_fg_counts(const unsigned long long *fg_count, int nsub, unsigned long long *packed) {
  for (int i = (int)(blockIdx.x * blockDim.x + threadIdx.x); i < nsub; i += (int)(gridDim.x * blockDim.x))
    packed[i] = fg_count[(int64_t)i * kFgCountStride];
}

void pack_fg_counts_async(const unsigned long long *fg_count, int nsub, unsigned long long *packed, cudaStream_t s) {
  if (nsub > 0)
    KLAUNCH("k_pack_fg_counts", s, (k_pack_fg_counts<<<std::min<unsigned>(ceil_div(nsub, 256), 64u), 256, 0, s>>>(
                                       fg_count, nsub, packed)));
}

// ------------------------------------------------------------------ launchers
void launch_scan(const ScanSeg &sg, int nsub, const uint32_t *in, uint32_t *out, uint32_t *chunk,
                 int64_t *totals, int64_t add, cudaStream_t s) {
  const unsigned nch = ceil_div(sg.max_len, 1024);
  KLAUNCH("k_scan_p1", s, (k_scan_p1<<<dim3(nch, nsub), 1024, 0, s>>>(sg.off, sg.len, sg.chk, in, chunk)));
  KLAUNCH("k_scan_p2", s, (k_scan_p2<<<nsub, 1024, 0, s>>>(sg.len, sg.chk, chunk, totals, add)));
  KLAUNCH("k_scan_p3", s, (k_scan_p3<<<dim3(nch, nsub), 1024, 0, s>>>(sg.off, sg.len, sg.chk, in, chunk, out)));
}

void launch_regions(const Sub *d_subs, int nsub, int64_t max_n, const ScanSeg &vseg, const uint8_t *mask,
                    const int32_t *labels, const uint32_t *root_bits, const float *norm, const float *dog,
                    int32_t *rank, uint32_t *blk_counts, uint32_t *blk_offsets, uint32_t *chunk,
                    int64_t *d_num_regions, RegionAcc acc, int64_t slots, int *d_status, cudaStream_t s) {
  launch_scan(vseg, nsub, blk_counts, blk_offsets, chunk, d_num_regions, 1, s);
  KLAUNCH("k_rank", s, (k_rank<<<dim3(ceil_div(max_n, kScanBlock), nsub), kRankThreads, 0, s>>>(d_subs, root_bits, blk_offsets, rank,
                                                                        acc, slots, d_status)));
  KLAUNCH("k_accumulate", s, (k_accumulate<<<dim3(ceil_div(max_n, kScanBlock), nsub), 256, 0, s>>>(d_subs, mask, labels, rank, norm, dog, acc,
                                                                slots)));
}

void launch_regions_fg(const Sub *d_subs, int nsub, int64_t max_n, int64_t max_fg, const ScanSeg &vseg,
                       const int32_t *fg_root, const uint32_t *root_bits, const FgEntry *fg,
                       const unsigned long long *fg_count, int32_t *rank, uint32_t *blk_counts,
                       uint32_t *blk_offsets, uint32_t *chunk, int64_t *d_num_regions, RegionAcc acc, int64_t slots,
                       int *d_status, int num_sms, cudaStream_t s) {
  launch_scan(vseg, nsub, blk_counts, blk_offsets, chunk, d_num_regions, 1, s);
  KLAUNCH("k_rank", s, (k_rank<<<dim3(ceil_div(max_n, kScanBlock), nsub), kRankThreads, 0, s>>>(d_subs, root_bits, blk_offsets,
                                                                                      rank, acc, slots, d_status)));
  int64_t want = (int64_t)ceil_div(max_fg, 8 * kAccSpan);   // eight warps of 256-thread blocks
  const int64_t cap = (int64_t)8 * num_sms / (nsub > 0 ? nsub : 1) + 1;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  const unsigned blocks = (unsigned)want;
  KLAUNCH("k_accumulate_fg", s, (k_accumulate_fg<<<dim3(blocks, nsub), 256, 0, s>>>(d_subs, fg, fg_count, fg_root,
                                                                                    rank, acc, slots)));
}

void launch_finalize(const Sub *d_subs, int nsub, int64_t max_reg_cap, const ScanSeg &rseg,
                     const int64_t *d_num_regions, RegionAcc acc, int64_t slots, RegionOut out,
                     FilterParams fp, uint32_t *blk_counts, uint32_t *blk_offsets, uint32_t *chunk,
                     int64_t *d_num_records, hdog_record *records, int64_t blk_stride, cudaStream_t s) {
  // the kernels visit only the blocks that hold regions (the count is on the device): the
  // other blocks' counts are zero for the record scan
  const int64_t nb = ceil_div(max_reg_cap, kFinalizeBlock);
  zero_async(blk_counts, (size_t)((nsub - 1) * blk_stride + nb) * sizeof(uint32_t), s);
  const unsigned grid = (unsigned)std::min<int64_t>(nb, 2048);
  KLAUNCH("k_finalize", s, (k_finalize<<<dim3(grid, nsub), kFinalizeBlock, 0, s>>>(d_subs, d_num_regions, acc, slots, out, fp, blk_counts)));
  launch_scan(rseg, nsub, blk_counts, blk_offsets, chunk, d_num_records, 0, s);
  KLAUNCH("k_records", s, (k_records<<<dim3(grid, nsub), kFinalizeBlock, 0, s>>>(d_subs, d_num_regions, out, acc.count, slots, blk_offsets,
                                                      records)));
}

}  // namespace hdog
