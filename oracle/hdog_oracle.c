/*
 * hdog_oracle.c -- TEST INFRASTRUCTURE ONLY (the parity checker, never the product).
 *
 * A CPU restatement of the reference HDoG cell-candidate chain of CUBIC-informatics,
 * src/3D.  Every float operation is written in the order the reference kernels perform
 * it, so that the restatement reproduces the reference FP32 path bit for bit:
 *   - sums are sequential in the reference's tap order and start from 0.0f;
 *   - the Gaussian convolution accumulates `sum += k * s` as an FMA chain (fmaf), the form
 *     nvcc gives `sum += a * b` under its default -fmad=true;
 *   - the Sylvester test comes in several contraction forms (pd_variant) so the form the
 *     reference binary uses can be pinned against it;
 *   - no fast-math, no flush-to-zero; the file is compiled with -ffp-contract=off so the
 *     compiler adds no contractions of its own on any host.
 * Region float sums are the one place the reference's order is set by CUB's
 * ReduceByKey (src/3D/RegionalFeatures.cu:295-329); the restatement keeps both a
 * sequential float sum in voxel order and a double sum, and tests compare within a
 * stated tolerance there.
 */
#include "hdog_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline uint16_t minu16(uint16_t a, uint16_t b) { return b < a ? b : a; }
static inline uint16_t maxu16(uint16_t a, uint16_t b) { return b > a ? b : a; }

/* calcGaussianWeight, src/3D/DoG3DFilter.cu:372-392 (TRUNCATE 2.0, MAX_KERNEL_LENGTH 80). */
int orc_gauss_taps(float sigma, float *h) {
  int lw = (int)(2.0 * sigma + 0.5);
  int length = lw * 2 + 1;
  float p, sum;
  sum = 1.f;
  h[lw] = 1.f;
  sigma *= sigma;
  for (int i = 1; i <= lw; i++) {
    p = (float)exp(-0.5 * i * i / sigma);
    h[lw - i] = p;
    h[lw + i] = p;
    sum += p * 2;
  }
  for (int i = 0; i < length; i++) h[i] /= sum;
  for (int i = length; i < ORC_MAX_TAPS; i++) h[i] = 0;
  return lw;
}

/* DoG3DFilter normalizer, src/3D/DoG3DFilter.cu:432. */
float orc_dog_normalizer(float sxy1, float sz1, float gamma) {
  return powf(sxy1, gamma * 2) * powf(sz1, gamma);
}

/* ---------------- normalization (src/3D/NormalizeFilter.cu) ---------------- */

/* Separable running min/max with nearest-edge borders, passes x -> y -> z
   (minmaxRows3DKernel :293-345, minmaxColumns3DKernel :374-425, minmaxLayers3DKernel
   :453-506; ErosionLarge3DFilter / DilationLarge3DFilter :549-569).  Min and max are
   exact, so only the border rule and the window matter. */
static void minmax_pass_x(const uint16_t *src, uint16_t *dst, int W, int H, int D, int r, int is_min) {
#pragma omp parallel for
  for (int z = 0; z < D; z++) {
    uint16_t *buf = (uint16_t *)malloc((size_t)(W + 2 * r) * sizeof(uint16_t));
    for (int y = 0; y < H; y++) {
      const uint16_t *row = src + ((size_t)z * H + y) * W;
      uint16_t *out = dst + ((size_t)z * H + y) * W;
      for (int i = 0; i < W + 2 * r; i++) buf[i] = row[clampi(i - r, 0, W - 1)];
      for (int x = 0; x < W; x++) out[x] = buf[x];
      for (int j = 1; j <= 2 * r; j++) {
        if (is_min) for (int x = 0; x < W; x++) out[x] = minu16(out[x], buf[x + j]);
        else for (int x = 0; x < W; x++) out[x] = maxu16(out[x], buf[x + j]);
      }
    }
    free(buf);
  }
}

static void minmax_pass_y(const uint16_t *src, uint16_t *dst, int W, int H, int D, int r, int is_min) {
#pragma omp parallel for
  for (int z = 0; z < D; z++) {
    for (int y = 0; y < H; y++) {
      uint16_t *out = dst + ((size_t)z * H + y) * W;
      const uint16_t *first = src + ((size_t)z * H + clampi(y - r, 0, H - 1)) * W;
      for (int x = 0; x < W; x++) out[x] = first[x];
      for (int j = 1; j <= 2 * r; j++) {
        const uint16_t *row = src + ((size_t)z * H + clampi(y - r + j, 0, H - 1)) * W;
        if (is_min) for (int x = 0; x < W; x++) out[x] = minu16(out[x], row[x]);
        else for (int x = 0; x < W; x++) out[x] = maxu16(out[x], row[x]);
      }
    }
  }
}

static void minmax_pass_z(const uint16_t *src, uint16_t *dst, int W, int H, int D, int r, int is_min) {
  const size_t plane = (size_t)W * H;
#pragma omp parallel for
  for (int z = 0; z < D; z++) {
    uint16_t *out = dst + (size_t)z * plane;
    const uint16_t *first = src + (size_t)clampi(z - r, 0, D - 1) * plane;
    memcpy(out, first, plane * sizeof(uint16_t));
    for (int j = 1; j <= 2 * r; j++) {
      const uint16_t *sl = src + (size_t)clampi(z - r + j, 0, D - 1) * plane;
      if (is_min) for (size_t i = 0; i < plane; i++) out[i] = minu16(out[i], sl[i]);
      else for (size_t i = 0; i < plane; i++) out[i] = maxu16(out[i], sl[i]);
    }
  }
}

void orc_minmax3d_nearest(const uint16_t *src, uint16_t *ero, uint16_t *dil, int W, int H, int D,
                          int rxy, int rz) {
  size_t n = (size_t)W * H * D;
  uint16_t *t = (uint16_t *)malloc(n * sizeof(uint16_t));
  if (ero) {
    minmax_pass_x(src, ero, W, H, D, rxy, 1);
    minmax_pass_y(ero, t, W, H, D, rxy, 1);
    minmax_pass_z(t, ero, W, H, D, rz, 1);
  }
  if (dil) {
    minmax_pass_x(src, dil, W, H, D, rxy, 0);
    minmax_pass_y(dil, t, W, H, D, rxy, 0);
    minmax_pass_z(t, dil, W, H, D, rz, 0);
  }
  free(t);
}

/* Box mean with nearest-edge borders: `val = 0; for j in 0..2r: val += s[j]; out = val *
   (1.0f/(2r+1))`, passes x -> y -> z (uniformRows3DKernel :55-105, uniformColumns3DKernel
   :134-183, uniformLayers3DKernel :211-262; UniformLarge3DFilter :537-546). */
void orc_box3d_nearest(const uint16_t *src, float *dst, int W, int H, int D, int rxy, int rz) {
  const size_t plane = (size_t)W * H, n = plane * D;
  float *t = (float *)malloc(n * sizeof(float));
  const float inv_xy = 1.0f / (2 * rxy + 1);
  const float inv_z = 1.0f / (2 * rz + 1);
  /* x: uint16 -> float */
#pragma omp parallel for
  for (int z = 0; z < D; z++) {
    float *buf = (float *)malloc((size_t)(W + 2 * rxy) * sizeof(float));
    float *acc = (float *)malloc((size_t)W * sizeof(float));
    for (int y = 0; y < H; y++) {
      const uint16_t *row = src + ((size_t)z * H + y) * W;
      for (int i = 0; i < W + 2 * rxy; i++) buf[i] = (float)row[clampi(i - rxy, 0, W - 1)];
      for (int x = 0; x < W; x++) acc[x] = 0.0f;
      for (int j = 0; j <= 2 * rxy; j++)
        for (int x = 0; x < W; x++) acc[x] += buf[x + j];
      float *out = dst + ((size_t)z * H + y) * W;
      for (int x = 0; x < W; x++) out[x] = acc[x] * inv_xy;
    }
    free(buf);
    free(acc);
  }
  /* y */
#pragma omp parallel for
  for (int z = 0; z < D; z++) {
    float *acc = (float *)malloc((size_t)W * sizeof(float));
    for (int y = 0; y < H; y++) {
      for (int x = 0; x < W; x++) acc[x] = 0.0f;
      for (int j = 0; j <= 2 * rxy; j++) {
        const float *row = dst + ((size_t)z * H + clampi(y - rxy + j, 0, H - 1)) * W;
        for (int x = 0; x < W; x++) acc[x] += row[x];
      }
      float *out = t + ((size_t)z * H + y) * W;
      for (int x = 0; x < W; x++) out[x] = acc[x] * inv_xy;
    }
    free(acc);
  }
  /* z */
#pragma omp parallel for
  for (int z = 0; z < D; z++) {
    float *out = dst + (size_t)z * plane;
    for (size_t i = 0; i < plane; i++) out[i] = 0.0f;
    for (int j = 0; j <= 2 * rz; j++) {
      const float *sl = t + (size_t)clampi(z - rz + j, 0, D - 1) * plane;
      for (size_t i = 0; i < plane; i++) out[i] += sl[i];
    }
    for (size_t i = 0; i < plane; i++) out[i] = out[i] * inv_z;
  }
  free(t);
}

/* Normalize3DFilter, src/3D/NormalizeFilter.cu:603-654 (Normalize3DKernel :571-586,
   Copy3DKernel :588-601). */
void orc_normalize(const uint16_t *img, float *norm, int W, int H, int D, int rxy, int rz,
                   float min_intensity, float *ero_l, float *dil_l) {
  const size_t n = (size_t)W * H * D;
  if (rxy == 0 || rz == 0) {
#pragma omp parallel for
    for (long long i = 0; i < (long long)n; i++) {
      const float v = (float)img[i];
      norm[i] = (v >= min_intensity) ? v : 0;
    }
    return;
  }
  uint16_t *m = (uint16_t *)malloc(n * sizeof(uint16_t));
  float *e = ero_l ? ero_l : (float *)malloc(n * sizeof(float));
  float *d = dil_l ? dil_l : (float *)malloc(n * sizeof(float));
  orc_minmax3d_nearest(img, m, NULL, W, H, D, rxy, rz);
  orc_box3d_nearest(m, e, W, H, D, rxy, rz);
  orc_minmax3d_nearest(img, NULL, m, W, H, D, rxy, rz);
  orc_box3d_nearest(m, d, W, H, D, rxy, rz);
#pragma omp parallel for
  for (long long i = 0; i < (long long)n; i++) {
    const float v = (float)img[i];
    norm[i] = (v >= min_intensity) ? (v - e[i]) / (d[i] - e[i]) : 0;
  }
  free(m);
  if (!ero_l) free(e);
  if (!dil_l) free(d);
}

/* ---------------- DoG (src/3D/DoG3DFilter.cu) ---------------- */

/* Separable Gaussian with zero borders, x -> y -> z; each output is the FMA chain
   `sum = 0; for j = -r..r: sum = fma(k[r-j], s[x+j], sum)` (convolutionRows3DKernel
   :70-130, convolutionColumns3DKernel :165-221, convolutionLayers3DKernel :256-313). */
void orc_gauss3d(const float *src, float *dst, int W, int H, int D, const float *kxy, int rxy,
                 const float *kz, int rz) {
  const size_t plane = (size_t)W * H, n = plane * D;
  float *t = (float *)malloc(n * sizeof(float));
  /* x: src -> dst */
#pragma omp parallel for
  for (int z = 0; z < D; z++) {
    float *buf = (float *)malloc((size_t)(W + 2 * rxy) * sizeof(float));
    float *acc = (float *)malloc((size_t)W * sizeof(float));
    for (int y = 0; y < H; y++) {
      const float *row = src + ((size_t)z * H + y) * W;
      for (int i = 0; i < W + 2 * rxy; i++) {
        int xx = i - rxy;
        buf[i] = (xx >= 0 && xx < W) ? row[xx] : 0.0f;
      }
      for (int x = 0; x < W; x++) acc[x] = 0.0f;
      for (int j = -rxy; j <= rxy; j++) {
        const float k = kxy[rxy - j];
        for (int x = 0; x < W; x++) acc[x] = fmaf(k, buf[x + rxy + j], acc[x]);
      }
      memcpy(dst + ((size_t)z * H + y) * W, acc, (size_t)W * sizeof(float));
    }
    free(buf);
    free(acc);
  }
  /* y: dst -> t */
#pragma omp parallel for
  for (int z = 0; z < D; z++) {
    float *acc = (float *)malloc((size_t)W * sizeof(float));
    for (int y = 0; y < H; y++) {
      for (int x = 0; x < W; x++) acc[x] = 0.0f;
      for (int j = -rxy; j <= rxy; j++) {
        const float k = kxy[rxy - j];
        const int yy = y + j;
        if (yy >= 0 && yy < H) {
          const float *row = dst + ((size_t)z * H + yy) * W;
          for (int x = 0; x < W; x++) acc[x] = fmaf(k, row[x], acc[x]);
        } else {
          for (int x = 0; x < W; x++) acc[x] = fmaf(k, 0.0f, acc[x]);
        }
      }
      memcpy(t + ((size_t)z * H + y) * W, acc, (size_t)W * sizeof(float));
    }
    free(acc);
  }
  /* z: t -> dst */
#pragma omp parallel for
  for (int z = 0; z < D; z++) {
    float *out = dst + (size_t)z * plane;
    for (size_t i = 0; i < plane; i++) out[i] = 0.0f;
    for (int j = -rz; j <= rz; j++) {
      const float k = kz[rz - j];
      const int zz = z + j;
      if (zz >= 0 && zz < D) {
        const float *sl = t + (size_t)zz * plane;
        for (size_t i = 0; i < plane; i++) out[i] = fmaf(k, sl[i], out[i]);
      } else {
        for (size_t i = 0; i < plane; i++) out[i] = fmaf(k, 0.0f, out[i]);
      }
    }
  }
  free(t);
}

/* DoG3DFilter, src/3D/DoG3DFilter.cu:417-437: large sigma first, then small, then
   `(small - large) * normalizer` (NormalizeSubtract3DKernel :346-354). */
void orc_dog(const float *norm, float *dog, int W, int H, int D, float sxy1, float sz1,
             float sxy2, float sz2, float gamma) {
  float k[4][ORC_MAX_TAPS];
  int r[4];
  r[0] = orc_gauss_taps(sxy1, k[0]);
  r[1] = orc_gauss_taps(sz1, k[1]);
  r[2] = orc_gauss_taps(sxy2, k[2]);
  r[3] = orc_gauss_taps(sz2, k[3]);
  const float normalizer = orc_dog_normalizer(sxy1, sz1, gamma);
  const size_t n = (size_t)W * H * D;
  float *large = (float *)malloc(n * sizeof(float));
  orc_gauss3d(norm, large, W, H, D, k[2], r[2], k[3], r[3]);
  orc_gauss3d(norm, dog, W, H, D, k[0], r[0], k[1], r[1]);
#pragma omp parallel for
  for (long long i = 0; i < (long long)n; i++) dog[i] = (dog[i] - large[i]) * normalizer;
  free(large);
}

/* ---------------- Hessian + negative-definite test ---------------- */

/* Sylvester test of PositiveDefiniteKernel, src/3D/Hessian3DFilter_element.cu:295-323:
     xx < 0 && xx*yy - xy*xy > 0 &&
     xx*yy*zz + 2*xy*yz*xz - xx*yz*yz - yy*xz*xz - zz*xy*xy < 0
   The expression leaves the compiler free to contract products into FMAs and to fold
   `a - b > 0` into `a > b`; pd_variant names one combination so the form the
   reference binary uses can be pinned against it.
     bits 0-1, 2x2 minor:  0  both products rounded, then compared / subtracted
                           1  fma(xx, yy, -(xy*xy))
                           2  fma(-xy, xy, xx*yy)
     bits 2-4, determinant, with A = (xx*yy)*zz, B = ((2*xy)*yz)*xz, C = (xx*yz)*yz,
               D = (yy*xz)*xz, E = (zz*xy)*xy:
                           0  every product rounded, (((A + B) - C) - D) - E < 0
                           1  t = fma(xx*yy, zz, B); t = fma(-(xx*yz), yz, t);
                              t = fma(-(yy*xz), xz, t); fma(-(zz*xy), xy, t) < 0
                           2  as 1 with B fused first: t = fma((2*xy)*yz, xz, A)
                           3  as 1, the last subtraction folded into the compare: t < E
                           4  as 2, the last subtraction folded into the compare: t < E */
int orc_pd_test(float xx, float xy, float xz, float yy, float yz, float zz, int v) {
  if (!(xx < 0)) return 0;
  const int vm = v & 3, vd = (v >> 2) & 7;
  if (vm == 1) {
    if (!(fmaf(xx, yy, -(xy * xy)) > 0)) return 0;
  } else if (vm == 2) {
    if (!(fmaf(-xy, xy, xx * yy) > 0)) return 0;
  } else {
    const float a = xx * yy, b = xy * xy;
    if (!(a - b > 0)) return 0;
  }
  const float p = xx * yy;
  const float q = (2.0f * xy) * yz;
  if (vd == 0) {
    float A = p * zz, B = q * xz, C = (xx * yz) * yz, Dd = (yy * xz) * xz, E = (zz * xy) * xy;
    float s = A + B;
    s = s - C;
    s = s - Dd;
    return (s - E) < 0;
  }
  float t = (vd == 2 || vd == 4) ? fmaf(q, xz, p * zz) : fmaf(p, zz, q * xz);
  t = fmaf(-(xx * yz), yz, t);
  t = fmaf(-(yy * xz), xz, t);
  if (vd == 3 || vd == 4) return t < (zz * xy) * xy;
  return fmaf(-(zz * xy), xy, t) < 0;
}

void orc_pd_test_planes(const float *planes, int64_t n, int v, uint8_t *out) {
#pragma omp parallel for
  for (int64_t i = 0; i < n; i++)
    out[i] = (uint8_t)orc_pd_test(planes[i], planes[n + i], planes[2 * n + i], planes[3 * n + i], planes[4 * n + i],
                                  planes[5 * n + i], v);
}

/* One central difference with a zero halo, gradientRowsKernel :22-74 and its column /
   layer twins: `sum = 0; sum += s[+1]; sum -= s[-1]; sum *= 0.5f`. */
static inline float cdiff(float plus, float minus) {
  float s = 0.0f;
  s += plus;
  s -= minus;
  s *= 0.5f;
  return s;
}

static inline float dog_at(const float *f, int W, int H, int D, int x, int y, int z) {
  if (x < 0 || y < 0 || z < 0 || x >= W || y >= H || z >= D) return 0.0f;
  return f[((size_t)z * H + y) * W + x];
}

/* First derivative along axis a (0 x, 1 y, 2 z) at a voxel inside the volume. */
static inline float grad1(const float *f, int W, int H, int D, int x, int y, int z, int a) {
  if (x < 0 || y < 0 || z < 0 || x >= W || y >= H || z >= D) return 0.0f;
  int dx = a == 0, dy = a == 1, dz = a == 2;
  return cdiff(dog_at(f, W, H, D, x + dx, y + dy, z + dz), dog_at(f, W, H, D, x - dx, y - dy, z - dz));
}

/* The six Hessian elements at one voxel, HessianPositiveDefiniteWithElement
   (:355-388): Hxx = gx(gx(f)), Hxy = gy(gx(f)), Hxz = gz(gx(f)), Hyy = gy(gy(f)),
   Hyz = gz(gy(f)), Hzz = gz(gz(f)), each gradient with a zero halo. */
void orc_hessian_at(const float *f, int W, int H, int D, int x, int y, int z, float o[6]) {
  o[0] = cdiff(grad1(f, W, H, D, x + 1, y, z, 0), grad1(f, W, H, D, x - 1, y, z, 0));
  o[1] = cdiff(grad1(f, W, H, D, x, y + 1, z, 0), grad1(f, W, H, D, x, y - 1, z, 0));
  o[2] = cdiff(grad1(f, W, H, D, x, y, z + 1, 0), grad1(f, W, H, D, x, y, z - 1, 0));
  o[3] = cdiff(grad1(f, W, H, D, x, y + 1, z, 1), grad1(f, W, H, D, x, y - 1, z, 1));
  o[4] = cdiff(grad1(f, W, H, D, x, y, z + 1, 1), grad1(f, W, H, D, x, y, z - 1, 1));
  o[5] = cdiff(grad1(f, W, H, D, x, y, z + 1, 2), grad1(f, W, H, D, x, y, z - 1, 2));
}

void orc_hessian_pd(const float *dog, uint8_t *mask, float *hess6, int W, int H, int D, int v) {
  const size_t n = (size_t)W * H * D;
#pragma omp parallel for
  for (int z = 0; z < D; z++) {
    for (int y = 0; y < H; y++) {
      for (int x = 0; x < W; x++) {
        float h[6];
        orc_hessian_at(dog, W, H, D, x, y, z, h);
        size_t i = ((size_t)z * H + y) * W + x;
        if (hess6)
          for (int k = 0; k < 6; k++) hess6[k * n + i] = h[k];
        mask[i] = (uint8_t)orc_pd_test(h[0], h[1], h[2], h[3], h[4], h[5], v);
      }
    }
  }
}

/* ---------------- CCL (src/3D/CCL3D.cu) ---------------- */

static inline int32_t uf_find(int32_t *p, int32_t a) {
  while (p[a] != a) {
    p[a] = p[p[a]];
    a = p[a];
  }
  return a;
}

/* Final labels of the reference's label-equivalence CCL (CCL3D.cu:17-117).  Label i
   starts as i*mask[i], so voxel 0 is background; neighbours are the 26 LINEAR offsets
   dz*W*H + dy*W + dx kept only when inside [0, N), which wraps across row and slice
   ends.  The iteration's fixed point gives every component the minimum linear index of
   its voxels; a sequential union-find over the same graph, always hanging the larger
   root under the smaller, gives the same labels.  Returns the region count, background
   included. */
int64_t orc_ccl(const uint8_t *mask, int32_t *lab, int W, int H, int D) {
  const int64_t n = (int64_t)W * H * D;
  int64_t offs[27];
  int no = 0;
  for (int dz = -1; dz <= 1; dz++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        int64_t o = (int64_t)dz * W * H + (int64_t)dy * W + dx;
        if (o >= 0) continue;
        int dup = 0;
        for (int k = 0; k < no; k++) dup |= offs[k] == o;
        if (!dup) offs[no++] = o;
      }
  for (int64_t i = 0; i < n; i++) lab[i] = (i > 0 && mask[i]) ? (int32_t)i : 0;
  for (int64_t i = 1; i < n; i++) {
    if (!lab[i]) continue;
    for (int k = 0; k < no; k++) {
      int64_t j = i + offs[k];
      if (j <= 0 || !lab[j]) continue;
      int32_t a = uf_find(lab, (int32_t)i), b = uf_find(lab, (int32_t)j);
      if (a == b) continue;
      if (a < b) lab[b] = a;
      else lab[a] = b;
    }
  }
  int64_t roots = 0;
  for (int64_t i = 1; i < n; i++) {
    if (!lab[i]) continue;
    lab[i] = uf_find(lab, (int32_t)i);
    roots += lab[i] == i;
  }
  return roots + 1;
}

/* ---------------- regional features (src/3D/RegionalFeatures.cu) ---------------- */

int orc_regions_compute(const int32_t *lab, const float *norm, const float *dog, int W, int H,
                        int D, orc_regions *o) {
  const int64_t n = (int64_t)W * H * D;
  int32_t *rank = (int32_t *)malloc((size_t)n * sizeof(int32_t));
  if (!rank) return -1;
  int64_t R = 1;
  for (int64_t i = 1; i < n; i++)
    if (lab[i] == i) rank[i] = (int32_t)R++;
  memset(o, 0, sizeof(*o));
  o->num_regions = R;
  o->label = (int32_t *)calloc(R, sizeof(int32_t));
  o->count = (int64_t *)calloc(R, sizeof(int64_t));
  o->max_norm = (float *)calloc(R, sizeof(float));
  o->sum_norm_f32 = (float *)calloc(R, sizeof(float));
  o->sum_norm_f64 = (double *)calloc(R, sizeof(double));
  o->sum_x = (double *)calloc(R, sizeof(double));
  o->sum_y = (double *)calloc(R, sizeof(double));
  o->sum_z = (double *)calloc(R, sizeof(double));
  o->hess_f32 = (float *)calloc(6 * R, sizeof(float));
  o->hess_f64 = (double *)calloc(6 * R, sizeof(double));
  for (int64_t i = 1; i < n; i++)
    if (lab[i] == i) o->label[rank[i]] = (int32_t)i;
  o->count[0] = 0;
  for (int64_t i = 0; i < n; i++) {
    if (!lab[i]) { o->count[0]++; continue; }
    const int64_t r = rank[lab[i]];
    const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)(i / ((int64_t)W * H));
    const float v = norm[i];
    if (o->count[r] == 0) o->max_norm[r] = v;
    else o->max_norm[r] = (v > o->max_norm[r]) ? v : o->max_norm[r];
    o->count[r]++;
    o->sum_norm_f32[r] += v;
    o->sum_norm_f64[r] += v;
    o->sum_x[r] += x;
    o->sum_y[r] += y;
    o->sum_z[r] += z;
    float h[6];
    orc_hessian_at(dog, W, H, D, x, y, z, h);
    for (int k = 0; k < 6; k++) {
      o->hess_f32[k * R + r] += h[k];
      o->hess_f64[k * R + r] += h[k];
    }
  }
  free(rank);
  return 0;
}

void orc_regions_free(orc_regions *r) {
  free(r->label); free(r->count); free(r->max_norm); free(r->sum_norm_f32); free(r->sum_norm_f64);
  free(r->sum_x); free(r->sum_y); free(r->sum_z); free(r->hess_f32); free(r->hess_f64);
  memset(r, 0, sizeof(*r));
}

/* EigenvaluesKernel<float>, src/3D/Eigenvalues.cu:19-96: Eberly's closed form for the
   symmetric 3x3 matrix of summed Hessian elements in double, structureness
   l0^2 + l1^2 + l2^2 and blobness l2^2 / (l0*l1), eigenvalues ascending. */
void orc_eigen(const float *hs, float *structureness, float *blobness) {
  double xx = hs[0], xy = hs[1], xz = hs[2], yy = hs[3], yz = hs[4], zz = hs[5];
  double max0 = fmax(fabs(xx), fabs(xy));
  double max1 = fmax(fabs(xz), fabs(yy));
  double max2 = fmax(fabs(yz), fabs(zz));
  double maxAbs = fmax(fmax(max0, max1), max2);
  if (maxAbs < 1e-30) {
    *structureness = 0;
    *blobness = 0;
    return;
  }
  double nrm = xy * xy + xz * xz + yz * yz;
  double e0, e1, e2;
  if (nrm > 1e-30) {
    double t = (xx + yy + zz) / 3.0;
    double b00 = xx - t, b11 = yy - t, b22 = zz - t;
    double den = sqrt((b00 * b00 + b11 * b11 + b22 * b22 + nrm * 2.0) / 6.0);
    double c00 = b11 * b22 - yz * yz;
    double c01 = xy * b22 - yz * xz;
    double c02 = xy * yz - b11 * xz;
    double det = (b00 * c00 - xy * c01 + xz * c02) / (den * den * den);
    double hd = det * 0.5;
    hd = fmin(fmax(hd, -1.0), 1.0);
    double ang = acos(hd) / 3.0;
    const double twoThirdsPi = 2.094395102393195;
    double beta2 = cos(ang) * 2.0;
    double beta0 = cos(ang + twoThirdsPi) * 2.0;
    double beta1 = -(beta0 + beta2);
    e0 = t + den * beta0;
    e1 = t + den * beta1;
    e2 = t + den * beta2;
  } else {
    e0 = xx; e1 = yy; e2 = zz;
  }
  *structureness = (float)(e0 * e0 + e1 * e1 + e2 * e2);
  double bd = e0 * e1;
  *blobness = (float)(e2 * e2 / bd);
}

/* ---------------- regional erosion (src/3D/Erosion3DFilter.cu) ---------------- */

/* Erosion3DFilter (:260-268): running min with a ZERO halo, x -> y -> z. */
void orc_erosion3d_zero(const uint16_t *src, uint16_t *dst, int W, int H, int D, int rxy, int rz) {
  const size_t plane = (size_t)W * H, n = plane * D;
  uint16_t *t = (uint16_t *)malloc(n * sizeof(uint16_t));
#pragma omp parallel for
  for (int z = 0; z < D; z++)
    for (int y = 0; y < H; y++)
      for (int x = 0; x < W; x++) {
        uint16_t m = 0xFFFF;
        for (int j = -rxy; j <= rxy; j++) {
          int xx = x + j;
          uint16_t v = (xx >= 0 && xx < W) ? src[((size_t)z * H + y) * W + xx] : 0;
          m = minu16(m, v);
        }
        dst[((size_t)z * H + y) * W + x] = m;
      }
#pragma omp parallel for
  for (int z = 0; z < D; z++)
    for (int y = 0; y < H; y++)
      for (int x = 0; x < W; x++) {
        uint16_t m = 0xFFFF;
        for (int j = -rxy; j <= rxy; j++) {
          int yy = y + j;
          uint16_t v = (yy >= 0 && yy < H) ? dst[((size_t)z * H + yy) * W + x] : 0;
          m = minu16(m, v);
        }
        t[((size_t)z * H + y) * W + x] = m;
      }
#pragma omp parallel for
  for (int z = 0; z < D; z++)
    for (size_t i = 0; i < plane; i++) {
      uint16_t m = 0xFFFF;
      for (int j = -rz; j <= rz; j++) {
        int zz = z + j;
        uint16_t v = (zz >= 0 && zz < D) ? t[(size_t)zz * plane + i] : 0;
        m = minu16(m, v);
      }
      dst[(size_t)z * plane + i] = m;
    }
  free(t);
}

/* ---------------- one substack end to end ---------------- */

/* processSubstack (src/3D/HDoG3D_main.cpp:134-257) plus saveFeatureVector
   (src/3D/utils.h:204-250).  img holds p->depth slices, the ones past depth_valid
   already zero. */
int64_t orc_substack(const orc_params *p, const uint16_t *img, int depth_valid, int z0,
                     orc_record *out, int64_t cap, int64_t *num_regions, uint8_t *mask_out,
                     int32_t *labels_out) {
  const int W = p->width, H = p->height, D = p->depth;
  const size_t n = (size_t)W * H * D;
  float *norm = (float *)malloc(n * sizeof(float));
  float *dog = (float *)malloc(n * sizeof(float));
  uint8_t *mask = mask_out ? mask_out : (uint8_t *)malloc(n);
  int32_t *lab = labels_out ? labels_out : (int32_t *)malloc(n * sizeof(int32_t));
  if (!norm || !dog || !mask || !lab) return -1;
  orc_normalize(img, norm, W, H, D, p->radius_norm_xy, p->radius_norm_z, p->min_intensity, NULL, NULL);
  orc_dog(norm, dog, W, H, D, p->sigma_xy_small, p->sigma_z_small, p->sigma_xy_large,
          p->sigma_z_large, p->gamma_n);
  orc_hessian_pd(dog, mask, NULL, W, H, D, p->pd_variant);
  orc_ccl(mask, lab, W, H, D);
  orc_regions r;
  orc_regions_compute(lab, norm, dog, W, H, D, &r);
  if (num_regions) *num_regions = r.num_regions;
  float taps[ORC_MAX_TAPS];
  const int depth_margin = orc_gauss_taps(p->sigma_z_large, taps) + p->extra_depth_margin;
  int64_t kept = 0;
  for (int64_t i = 1; i < r.num_regions; i++) {
    const uint16_t size16 = (uint16_t)(r.count[i] & 0xFFFF);
    const float cx = (float)r.sum_x[i] / (float)size16;
    const float cy = (float)r.sum_y[i] / (float)size16;
    const float cz = (float)r.sum_z[i] / (float)size16;
    if (cz < depth_margin || cz >= depth_valid - depth_margin) continue;
    if (cx < p->left_margin || cx >= W - p->right_margin) continue;
    if (cy < p->top_margin || cy >= H - p->bottom_margin) continue;
    const float intensity = p->is_ave_mode ? r.sum_norm_f32[i] : r.max_norm[i];
    if (size16 < p->min_size || intensity <= 0) continue;
    float hs[6], st, bl;
    for (int k = 0; k < 6; k++) hs[k] = r.hess_f32[k * r.num_regions + i];
    orc_eigen(hs, &st, &bl);
    if (kept < cap) {
      orc_record *rec = &out[kept];
      rec->centroid_x = cx;
      rec->centroid_y = cy;
      rec->centroid_z = cz + z0;
      rec->structureness = st;
      rec->blobness = bl;
      rec->intensity = intensity;
      rec->size = size16;
      rec->padding = 0;
    }
    kept++;
  }
  orc_regions_free(&r);
  free(norm);
  free(dog);
  if (!mask_out) free(mask);
  if (!labels_out) free(lab);
  return kept;
}
