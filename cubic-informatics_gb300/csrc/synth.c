/*
 * synth.c -- seeded synthetic light-sheet volumes for the HDoG benchmarks and tests.
 *
 * The reference publishes no dataset for the HDoG path, so every benchmark and parity
 * case runs on volumes made here: a uint16 background of mean 100 and s.d. 8 with
 * anisotropic Gaussian nuclei added on top, optionally with a linear z attenuation and
 * a per-slice, per-row gain ("striping").
 *
 * Determinism.  Every random quantity comes from a counter-based hash (splitmix64 of
 * seed, stream and counter), never from a sequential generator shared between
 * threads, so the volume is identical for any thread count.  The background noise is
 * an Irwin-Hall sum of twelve 16-bit uniforms, which is exact integer arithmetic, and
 * the only transcendental is the double-precision exp() of the nucleus profile.  The
 * file is built with -ffp-contract=off so that x86-64 and aarch64 hosts produce the
 * same volume bit for bit.
 *
 * Layout: img[(z*H + y)*W + x], x fastest, the raw slice layout HDoG3D_main reads
 * (src/3D/utils.h:160-173 in the reference).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "synth.h"

static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Hash of (seed, stream, counter): three rounds of splitmix64 finalisation. */
static inline uint64_t hash3(uint64_t seed, uint64_t stream, uint64_t ctr) {
  return mix64(mix64(mix64(seed) ^ (stream * 0xD1342543DE82EF95ull)) ^ ctr);
}

/* Uniform double in [0,1) with 53 random bits. */
static inline double unif(uint64_t seed, uint64_t stream, uint64_t ctr) {
  return (double)(hash3(seed, stream, ctr) >> 11) * (1.0 / 9007199254740992.0);
}

enum { ST_CENTRE = 1, ST_SHAPE = 2, ST_NOISE = 3, ST_STRIPE = 4, ST_PAIR = 5 };

/* Approximate N(0,1): Irwin-Hall sum of 12 uniform 16-bit integers, exact in double. */
static inline double gauss_voxel(uint64_t seed, uint64_t idx) {
  uint64_t s = 0;
  for (int k = 0; k < 3; k++) {
    uint64_t h = hash3(seed, ST_NOISE, idx * 3u + (uint64_t)k);
    s += (h & 0xFFFF) + ((h >> 16) & 0xFFFF) + ((h >> 32) & 0xFFFF) + (h >> 48);
  }
  return ((double)s - 393210.0) / 65536.0;
}

typedef struct {
  int *head;  /* per cell: first nucleus index, -1 when empty */
  int *next;  /* per nucleus: next index in the same cell */
  int gx, gy, gz;
  double cell;
} grid_t;

static int grid_cell(const grid_t *g, double x, double y, double z, int *cx, int *cy, int *cz) {
  *cx = (int)(x / g->cell); *cy = (int)(y / g->cell); *cz = (int)(z / g->cell);
  if (*cx >= g->gx) *cx = g->gx - 1;
  if (*cy >= g->gy) *cy = g->gy - 1;
  if (*cz >= g->gz) *cz = g->gz - 1;
  return (*cz * g->gy + *cy) * g->gx + *cx;
}

static int too_close(const grid_t *g, const hdog_nucleus *nu, double x, double y, double z, double sep) {
  int cx, cy, cz;
  grid_cell(g, x, y, z, &cx, &cy, &cz);
  for (int dz = -1; dz <= 1; dz++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        int ix = cx + dx, iy = cy + dy, iz = cz + dz;
        if (ix < 0 || iy < 0 || iz < 0 || ix >= g->gx || iy >= g->gy || iz >= g->gz) continue;
        for (int j = g->head[(iz * g->gy + iy) * g->gx + ix]; j >= 0; j = g->next[j]) {
          double ex = nu[j].x - x, ey = nu[j].y - y, ez = nu[j].z - z;
          if (ex * ex + ey * ey + ez * ez < sep * sep) return 1;
        }
      }
  return 0;
}

static void grid_add(grid_t *g, const hdog_nucleus *nu, int i) {
  int cx, cy, cz;
  int c = grid_cell(g, nu[i].x, nu[i].y, nu[i].z, &cx, &cy, &cz);
  g->next[i] = g->head[c];
  g->head[c] = i;
}

static void draw_shape(const hdog_synth_spec *s, uint64_t i, hdog_nucleus *n) {
  n->sigma_xy = s->sigma_xy_lo + (s->sigma_xy_hi - s->sigma_xy_lo) * unif(s->seed, ST_SHAPE, 4 * i + 0);
  n->sigma_z = s->sigma_z_lo + (s->sigma_z_hi - s->sigma_z_lo) * unif(s->seed, ST_SHAPE, 4 * i + 1);
  n->peak = s->peak_lo + (s->peak_hi - s->peak_lo) * unif(s->seed, ST_SHAPE, 4 * i + 2);
}

int64_t hdog_synth_nuclei(const hdog_synth_spec *s, hdog_nucleus *out, int64_t cap) {
  if (!s || !out || s->width <= 0 || s->height <= 0 || s->depth <= 0 || s->n_nuclei < 0) return -1;
  int64_t n_target = s->n_nuclei < cap ? s->n_nuclei : cap;
  int64_t n_pairs = (int64_t)(s->n_nuclei * s->pair_fraction / 2.0 + 0.5);
  if (2 * n_pairs > n_target) n_pairs = n_target / 2;
  int64_t n_primary = n_target - n_pairs;

  grid_t g;
  g.cell = s->min_separation > 1.0 ? s->min_separation : 1.0;
  g.gx = (int)(s->width / g.cell) + 1;
  g.gy = (int)(s->height / g.cell) + 1;
  g.gz = (int)(s->depth / g.cell) + 1;
  size_t ncell = (size_t)g.gx * g.gy * g.gz;
  g.head = (int *)malloc(ncell * sizeof(int));
  g.next = (int *)malloc((size_t)(n_target > 0 ? n_target : 1) * sizeof(int));
  if (!g.head || !g.next) { free(g.head); free(g.next); return -1; }
  for (size_t c = 0; c < ncell; c++) g.head[c] = -1;

  int64_t n = 0;
  uint64_t attempt = 0;
  for (int64_t i = 0; i < n_primary; i++) {
    double x = 0, y = 0, z = 0;
    for (int tries = 0; tries < 64; tries++, attempt++) {
      x = s->width * unif(s->seed, ST_CENTRE, 3 * attempt + 0);
      y = s->height * unif(s->seed, ST_CENTRE, 3 * attempt + 1);
      z = s->depth * unif(s->seed, ST_CENTRE, 3 * attempt + 2);
      if (s->min_separation <= 0 || !too_close(&g, out, x, y, z, s->min_separation)) break;
    }
    out[n].x = x; out[n].y = y; out[n].z = z;
    draw_shape(s, (uint64_t)n, &out[n]);
    grid_add(&g, out, (int)n);
    n++;
  }
  /* Touching pairs: the first n_pairs primaries each get a partner at centre distance
     pair_distance_factor * (sigma_xy1 + sigma_xy2) along a uniform random direction. */
  for (int64_t p = 0; p < n_pairs && n < n_target; p++) {
    const hdog_nucleus *a = &out[p];
    hdog_nucleus b;
    draw_shape(s, (uint64_t)n, &b);
    double cz = 2.0 * unif(s->seed, ST_PAIR, 2 * (uint64_t)p) - 1.0;
    double ph = 6.283185307179586 * unif(s->seed, ST_PAIR, 2 * (uint64_t)p + 1);
    double rxy = sqrt(1.0 - cz * cz);
    double d = s->pair_distance_factor * (a->sigma_xy + b.sigma_xy);
    b.x = a->x + d * rxy * cos(ph);
    b.y = a->y + d * rxy * sin(ph);
    b.z = a->z + d * cz;
    out[n++] = b;
  }
  free(g.head);
  free(g.next);
  return n;
}

int hdog_synth_render(const hdog_synth_spec *s, const hdog_nucleus *nu, int64_t n_nuclei,
                      int z_begin, int z_end, uint16_t *img) {
  if (!s || !img || z_begin < 0 || z_end > s->depth || z_begin > z_end) return -1;
  const int W = s->width, H = s->height, Z = s->depth;
  const size_t plane = (size_t)W * H;
  int rc = 0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int z = z_begin; z < z_end; z++) {
    double *acc = (double *)malloc(plane * sizeof(double));
    if (!acc) { rc = -1; continue; }
    uint16_t *dst = img + (size_t)(z - z_begin) * plane;
    for (size_t i = 0; i < plane; i++)
      acc[i] = s->bg_mean + s->bg_sd * gauss_voxel(s->seed, (uint64_t)z * plane + i);
    for (int64_t k = 0; k < n_nuclei; k++) {
      const hdog_nucleus *q = &nu[k];
      double ext_z = 3.0 * q->sigma_z + 1.0;
      double dz = (double)z - q->z;
      if (dz < -ext_z || dz > ext_z) continue;
      double ext = 3.0 * q->sigma_xy + 1.0;
      int x0 = (int)floor(q->x - ext), x1 = (int)ceil(q->x + ext);
      int y0 = (int)floor(q->y - ext), y1 = (int)ceil(q->y + ext);
      if (x0 < 0) x0 = 0;
      if (y0 < 0) y0 = 0;
      if (x1 > W - 1) x1 = W - 1;
      if (y1 > H - 1) y1 = H - 1;
      double ixy = 1.0 / (q->sigma_xy * q->sigma_xy), iz = 1.0 / (q->sigma_z * q->sigma_z);
      double ez = dz * dz * iz;
      for (int y = y0; y <= y1; y++) {
        double dy = (double)y - q->y;
        double ey = dy * dy * ixy + ez;
        double *row = acc + (size_t)y * W;
        for (int x = x0; x <= x1; x++) {
          double dx = (double)x - q->x;
          row[x] += q->peak * exp(-0.5 * (dx * dx * ixy + ey));
        }
      }
    }
    double att = 1.0;
    if (Z > 1) att = 1.0 + (s->atten_z_end - 1.0) * ((double)z / (double)(Z - 1));
    for (int y = 0; y < H; y++) {
      double gain = att;
      if (s->stripe_amplitude > 0)
        gain = att * (1.0 + s->stripe_amplitude * (2.0 * unif(s->seed, ST_STRIPE, (uint64_t)z * H + y) - 1.0));
      for (int x = 0; x < W; x++) {
        double v = floor(acc[(size_t)y * W + x] * gain + 0.5);
        if (v < 0) v = 0;
        if (v > 65535) v = 65535;
        dst[(size_t)y * W + x] = (uint16_t)v;
      }
    }
    free(acc);
  }
  return rc;
}

void hdog_synth_default_spec(hdog_synth_spec *s, int width, int height, int depth, int n_nuclei,
                             uint64_t seed) {
  memset(s, 0, sizeof(*s));
  s->width = width; s->height = height; s->depth = depth;
  s->n_nuclei = n_nuclei; s->seed = seed;
  s->bg_mean = 100.0; s->bg_sd = 8.0;
  s->sigma_xy_lo = 2.0; s->sigma_xy_hi = 3.5;
  s->sigma_z_lo = 1.2; s->sigma_z_hi = 2.0;
  s->peak_lo = 300.0; s->peak_hi = 3000.0;
  s->min_separation = 8.0;
  s->pair_fraction = 0.0; s->pair_distance_factor = 0.8;
  s->atten_z_end = 1.0; s->stripe_amplitude = 0.0;
}
