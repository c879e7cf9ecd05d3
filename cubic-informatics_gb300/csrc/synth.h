/* synth.h -- seeded synthetic volumes for HDoG benchmarks and tests (host C). */
#ifndef HDOG_SYNTH_H
#define HDOG_SYNTH_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int width, height, depth;      /* volume extent in voxels (x, y, z) */
  int n_nuclei;                  /* total nuclei, pairs included */
  uint64_t seed;
  double bg_mean, bg_sd;         /* background level and noise s.d. */
  double sigma_xy_lo, sigma_xy_hi, sigma_z_lo, sigma_z_hi;  /* nucleus s.d., voxels */
  double peak_lo, peak_hi;       /* nucleus peak amplitude */
  double min_separation;         /* rejection distance between centres (0 = none) */
  double pair_fraction;          /* fraction of nuclei placed in touching pairs */
  double pair_distance_factor;   /* pair centre distance = factor * (sxy1 + sxy2) */
  double atten_z_end;            /* gain at the last slice; linear from 1.0 at z=0 */
  double stripe_amplitude;       /* per-slice per-row gain 1 +/- amplitude */
} hdog_synth_spec;

typedef struct {
  double x, y, z, sigma_xy, sigma_z, peak;
} hdog_nucleus;

void hdog_synth_default_spec(hdog_synth_spec *s, int width, int height, int depth, int n_nuclei,
                             uint64_t seed);
/* Places nuclei; returns the count written (<= cap) or -1. */
int64_t hdog_synth_nuclei(const hdog_synth_spec *s, hdog_nucleus *out, int64_t cap);
/* Renders slices [z_begin, z_end) of the volume into img (slice z_begin first). */
int hdog_synth_render(const hdog_synth_spec *s, const hdog_nucleus *nu, int64_t n_nuclei,
                      int z_begin, int z_end, uint16_t *img);

#ifdef __cplusplus
}
#endif
#endif
