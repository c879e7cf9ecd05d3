// records.cu -- per-record steps after the HDoG records, sm_103a: local -> global
// coordinates, the scale-merge validity test and the classifier features.
//
// Reference (all NumPy on the host): script/HalfBrainCells.py:44-56 (HDoGResultStack),
// script/MergeBrain.py:546-570 (process_stack of the scale merge),
// script/HDoG_classifier.py:158-176 (get_X_3d).  One thread per record; every rounding
// step is an explicit round-to-nearest operation, so the compiler cannot contract a
// multiply and an add that NumPy rounds separately.
#include <cmath>

#include "kernels.cuh"

namespace hdog {

static_assert(sizeof(hdog_global) == 15 && sizeof(hdog_scalemerged) == 13, "packed NumPy record layouts");
static_assert(sizeof(hdog_global_params) == 72 && sizeof(hdog_scalemerge_params) == 184 &&
                  sizeof(hdog_clf_params) == 80,
              "parameter blocks as the bindings lay them out");

// offset + product: a float64 scalar against a float32 array (see HDOG_PROMOTE_*).
__device__ __forceinline__ float add_offset(double offset, float v, int promote) {
  return promote == HDOG_PROMOTE_F64 ? __double2float_rn(__dadd_rn(offset, (double)v))
                                     : __fadd_rn(__double2float_rn(offset), v);
}

__global__ void k_to_global(const hdog_record *rec, int64_t n, hdog_global_params p, hdog_global *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const hdog_record r = rec[i];
  // local * scale: the scale is a Python float, so NumPy multiplies in float32
  float gx = add_offset(p.offset_x, __fmul_rn(r.centroid_x, __double2float_rn(p.scale_x)), p.promote);
  float gy = add_offset(p.offset_y, __fmul_rn(r.centroid_y, __double2float_rn(p.scale_y)), p.promote);
  const float gz = add_offset(p.offset_z, __fmul_rn(r.centroid_z, __double2float_rn(p.scale_z)), p.promote);
  // flip: merged -= width * scale, a Python float subtracted in place from float32
  if (p.scale_x < 0) gx = __fsub_rn(gx, __double2float_rn(__dmul_rn((double)p.width, p.scale_x)));
  if (p.scale_y < 0) gy = __fsub_rn(gy, __double2float_rn(__dmul_rn((double)p.height, p.scale_y)));
  hdog_global g;
  g.merged_x = gx;
  g.merged_y = gy;
  g.merged_z = gz;
  g.i_x = (uint8_t)p.i_x;
  g.i_y = (uint8_t)p.i_y;
  g.fwrv = p.is_fw ? 0 : 1;
  // 15-byte records: byte stores keep every access aligned
  const uint8_t *src = reinterpret_cast<const uint8_t *>(&g);
  uint8_t *dst = reinterpret_cast<uint8_t *>(out + i);
#pragma unroll
  for (int k = 0; k < (int)sizeof(hdog_global); k++) dst[k] = src[k];
}

// (merged - offset) * coeff - margin, stored into a float32 array.
__device__ __forceinline__ float scaled_axis(float m, double offset, double coeff, double margin, int promote) {
  if (promote == HDOG_PROMOTE_F64)
    return __double2float_rn(__dsub_rn(__dmul_rn(__dsub_rn((double)m, offset), coeff), margin));
  const float t = __fsub_rn(m, __double2float_rn(offset));
  return __fsub_rn(__fmul_rn(t, __double2float_rn(coeff)), __double2float_rn(margin));
}

__global__ void k_scale_merge(const hdog_global *in, int64_t n, hdog_scalemerge_params p, hdog_scalemerged *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  hdog_global g;
  const uint8_t *src = reinterpret_cast<const uint8_t *>(in + i);
  uint8_t *gb = reinterpret_cast<uint8_t *>(&g);
#pragma unroll
  for (int k = 0; k < (int)sizeof(hdog_global); k++) gb[k] = src[k];
  const double lo = fmin(p.bound_z0, p.bound_z1), hi = fmax(p.bound_z0, p.bound_z1);
  bool valid;
  if (p.promote == HDOG_PROMOTE_F64)
    valid = lo <= (double)g.merged_z && (double)g.merged_z <= hi;
  else
    valid = __double2float_rn(lo) <= g.merged_z && g.merged_z <= __double2float_rn(hi);
  const float c[3] = {scaled_axis(g.merged_x, p.offset_x, p.coeff_x, p.margin_left, p.promote),
                      scaled_axis(g.merged_y, p.offset_y, p.coeff_y, p.margin_top, p.promote),
                      scaled_axis(g.merged_z, p.offset_z, p.coeff_z, 0.0, p.promote)};
  // A . c + b in float64 (A's entries are 0 or +-1, so the products are exact), then float32
  float s[3];
#pragma unroll
  for (int r = 0; r < 3; r++) {
    double acc = __dmul_rn(p.A[3 * r], (double)c[0]);
    acc = __dadd_rn(acc, __dmul_rn(p.A[3 * r + 1], (double)c[1]));
    acc = __dadd_rn(acc, __dmul_rn(p.A[3 * r + 2], (double)c[2]));
    s[r] = __double2float_rn(__dadd_rn(acc, p.b[r]));
  }
  hdog_scalemerged o;
  o.scaled_x = s[0];
  o.scaled_y = s[1];
  o.scaled_z = s[2];
  o.is_valid = valid ? 1 : 0;
  const uint8_t *ob = reinterpret_cast<const uint8_t *>(&o);
  uint8_t *dst = reinterpret_cast<uint8_t *>(out + i);
#pragma unroll
  for (int k = 0; k < (int)sizeof(hdog_scalemerged); k++) dst[k] = ob[k];
}

// numpy.nan_to_num: NaN -> 0, +-inf -> +-DBL_MAX.
__device__ __forceinline__ double nan_to_num(double v) {
  if (isnan(v)) return 0.0;
  if (isinf(v)) return v > 0 ? 1.7976931348623157e308 : -1.7976931348623157e308;
  return v;
}

__global__ void k_clf_features(const hdog_record *rec, int64_t n, hdog_clf_params p, double *X) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const hdog_record r = rec[i];
  // intensity / size is float32 / uint16 -> float32 in NumPy
  const float f[3] = {p.is_ave ? __fdiv_rn(r.intensity, (float)r.size) : r.intensity, r.structureness, r.blobness};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double v = __dmul_rn(__dadd_rn(log10(__dadd_rn((double)f[k], p.bias_before_log[k])), p.bias[k]), p.scale[k]);
    X[3 * i + k] = nan_to_num(v);
  }
}

void launch_to_global(const hdog_record *rec, int64_t n, const hdog_global_params &p, hdog_global *out,
                      cudaStream_t s) {
  if (n <= 0) return;
  KLAUNCH("k_to_global", s, (k_to_global<<<ceil_div(n, 256), 256, 0, s>>>(rec, n, p, out)));
}

void launch_scale_merge(const hdog_global *in, int64_t n, const hdog_scalemerge_params &p, hdog_scalemerged *out,
                        cudaStream_t s) {
  if (n <= 0) return;
  KLAUNCH("k_scale_merge", s, (k_scale_merge<<<ceil_div(n, 256), 256, 0, s>>>(in, n, p, out)));
}

void launch_clf_features(const hdog_record *rec, int64_t n, const hdog_clf_params &p, double *X, cudaStream_t s) {
  if (n <= 0) return;
  KLAUNCH("k_clf_features", s, (k_clf_features<<<ceil_div(n, 256), 256, 0, s>>>(rec, n, p, X)));
}

}  // namespace hdog
