/*
 * hdog_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference HDoG chain (CUBIC-informatics src/3D), used by the
 * tests, the smoke check and the bench's CPU-baseline leg as the parity checker.  The
 * product never links or calls this code.
 */
#ifndef HDOG_ORACLE_H
#define HDOG_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_TAPS 80

/* 28-byte candidate record, layout of FeatureVector (src/3D/utils.h:188-197). */
typedef struct {
  float centroid_x, centroid_y, centroid_z;
  float structureness, blobness, intensity;
  uint16_t size, padding;
} orc_record;

typedef struct {
  int width, height, depth;          /* substack extent; depth = HDoG_param.depth */
  int radius_norm_xy, radius_norm_z;
  float min_intensity;
  float gamma_n;
  float sigma_xy_small, sigma_z_small, sigma_xy_large, sigma_z_large;
  int left_margin, right_margin, top_margin, bottom_margin;
  int extra_depth_margin;
  int min_size;
  int is_ave_mode;
  int pd_variant;                    /* floating-point contraction form of the PD test */
} orc_params;

/* Per-region features (region 0 = background). Arrays have num_regions entries. */
typedef struct {
  int64_t num_regions;
  int32_t *label;          /* root label (min linear index) */
  int64_t *count;          /* exact voxel count (the record stores count mod 65536) */
  float *max_norm;         /* max of normalized intensity, sequential in voxel order */
  float *sum_norm_f32;     /* sequential float sum (is_ave_mode) */
  double *sum_norm_f64;
  double *sum_x, *sum_y, *sum_z;    /* exact coordinate sums */
  float *hess_f32;         /* 6 x num_regions, sequential float sums in voxel order */
  double *hess_f64;        /* 6 x num_regions, double sums */
} orc_regions;

int orc_gauss_taps(float sigma, float *taps /* ORC_MAX_TAPS */);
float orc_dog_normalizer(float sigma_xy_small, float sigma_z_small, float gamma);

void orc_minmax3d_nearest(const uint16_t *src, uint16_t *ero, uint16_t *dil, int W, int H, int D,
                          int rxy, int rz);
void orc_box3d_nearest(const uint16_t *src, float *dst, int W, int H, int D, int rxy, int rz);
void orc_normalize(const uint16_t *img, float *norm, int W, int H, int D, int rxy, int rz,
                   float min_intensity, float *ero_l /* opt */, float *dil_l /* opt */);
void orc_gauss3d(const float *src, float *dst, int W, int H, int D, const float *kxy, int rxy,
                 const float *kz, int rz);
void orc_dog(const float *norm, float *dog, int W, int H, int D, float sxy1, float sz1,
             float sxy2, float sz2, float gamma);
void orc_hessian_pd(const float *dog, uint8_t *mask, float *hess6 /* opt, 6*N */, int W, int H,
                    int D, int pd_variant);
int orc_pd_test(float xx, float xy, float xz, float yy, float yz, float zz, int pd_variant);
void orc_pd_test_planes(const float *planes /* 6 x n */, int64_t n, int pd_variant, uint8_t *out);
void orc_hessian_at(const float *dog, int W, int H, int D, int x, int y, int z, float out[6]);
int64_t orc_ccl(const uint8_t *mask, int32_t *labels, int W, int H, int D);
int orc_regions_compute(const int32_t *labels, const float *norm, const float *dog, int W, int H,
                        int D, orc_regions *out);
void orc_regions_free(orc_regions *r);
void orc_eigen(const float *hess_sum6 /* xx,xy,xz,yy,yz,zz */, float *structureness,
               float *blobness);
void orc_erosion3d_zero(const uint16_t *src, uint16_t *dst, int W, int H, int D, int rxy, int rz);

/* Whole chain for one substack: img is depth x H x W (the zero tail already applied).
   Writes at most cap records; returns the number of records kept, or -1. The number of
   regions (background included) goes to *num_regions when non-NULL. */
int64_t orc_substack(const orc_params *p, const uint16_t *img, int depth_valid, int z0,
                     orc_record *out, int64_t cap, int64_t *num_regions, uint8_t *mask_out,
                     int32_t *labels_out);

#ifdef __cplusplus
}
#endif
#endif
