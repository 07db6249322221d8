/*
 * Seeded synthetic rotation sweeps: raw uint32 frames with a Poisson
 * background, 3-D Gaussian spots spanning several frames, and detector masks
 * written in as the masked sentinel 0xFFFFFFFF (the threshold has no separate
 * mask input: a pixel at or above 0xFFFFFFFE is masked, src/spots/dext.cc:40).
 *
 * Every random draw is a hash of (seed, frame, pixel, draw number), so a frame
 * is the same whatever the thread count. (Across machines the libm functions
 * used for the spot profiles may differ in a last bit; fixtures that must be
 * identical everywhere are committed as data rather than regenerated.)
 * Frames are made on demand, so a long sweep never has to sit in memory.
 *
 * This is input generation for tests and benchmarks, not part of the
 * threshold or labelling path.
 */
#include "synth.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct sf_synth {
  sf_synth_params p;
  size_t n_spots;
  float *sx, *sy, *sz, *sig_xy, *sig_z, *peak; /* sorted by sz */
  double sig_z_max;
};

static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Uniform in (0, 1), from the 53 high bits of a hash. */
static inline double uniform(uint64_t key, uint64_t draw) {
  const uint64_t h = mix64(key ^ mix64(draw + 0x632BE59BD9B4E019ull));
  return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

static uint32_t poisson(double lambda, uint64_t key) {
  if (lambda <= 0.0)
    return 0;
  if (lambda < 30.0) {
    /* Knuth: multiply uniforms until the product drops below e^-lambda. */
    const double limit = exp(-lambda);
    double product = uniform(key, 0);
    uint32_t k = 0;
    while (product > limit && k < 1000) {
      product *= uniform(key, k + 1);
      k++;
    }
    return k;
  }
  /* Large means: a rounded normal (Box-Muller) is close enough here. */
  const double u1 = uniform(key, 0), u2 = uniform(key, 1);
  const double n = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
  const double v = floor(lambda + sqrt(lambda) * n + 0.5);
  return v < 0.0 ? 0u : (uint32_t)v;
}

void sf_synth_default_params(sf_synth_params *p) {
  memset(p, 0, sizeof(*p));
  p->height = 1024;
  p->width = 1024;
  p->seed = 1;
  p->n_frames = 100;
  p->bg_edge = 0.5;
  p->bg_centre = 0.5;
  p->spots_per_frame = 200.0;
  p->sigma_xy_min = p->sigma_xy_max = 1.2;
  p->sigma_z_min = p->sigma_z_max = 0.8;
  p->peak_min = 50.0;
  p->peak_max = 2000.0;
}

static int cmp_z(const void *a, const void *b) {
  const float x = ((const float *)a)[0], y = ((const float *)b)[0];
  return (x > y) - (x < y);
}

sf_synth *sf_synth_open(const sf_synth_params *params) {
  if (!params || params->height == 0 || params->width == 0 ||
      params->n_frames <= 0)
    return NULL;
  sf_synth *s = (sf_synth *)calloc(1, sizeof(sf_synth));
  if (!s)
    return NULL;
  s->p = *params;
  const sf_synth_params *p = &s->p;
  /* A spot is visible on about 2.5 sigma_z * 2 frames; centres are spread
   * over the sweep plus a margin so the first and last frames are as full as
   * the rest. spots_per_frame is the mean number visible on one frame. */
  const double span = fmax(1.0, 5.0 * 0.5 * (p->sigma_z_min + p->sigma_z_max));
  const double margin = 3.0 * p->sigma_z_max + 1.0;
  const double zlo = -margin, zhi = (double)p->n_frames + margin;
  s->n_spots = (size_t)(p->spots_per_frame * (zhi - zlo) / span + 0.5);
  float *tmp = (float *)malloc(s->n_spots * 6 * sizeof(float) + 1);
  if (!tmp) {
    free(s);
    return NULL;
  }
  const uint64_t key = mix64(p->seed ^ 0x53500753ull);
  for (size_t i = 0; i < s->n_spots; i++) {
    float *t = tmp + 6 * i;
    t[0] = (float)(zlo + (zhi - zlo) * uniform(key, 6 * i + 0));
    t[1] = (float)(3.0 + (p->width - 6.0) * uniform(key, 6 * i + 1));
    t[2] = (float)(3.0 + (p->height - 6.0) * uniform(key, 6 * i + 2));
    t[3] = (float)(p->sigma_xy_min +
                   (p->sigma_xy_max - p->sigma_xy_min) * uniform(key, 6 * i + 3));
    t[4] = (float)(p->sigma_z_min +
                   (p->sigma_z_max - p->sigma_z_min) * uniform(key, 6 * i + 4));
    /* log-uniform peak */
    t[5] = (float)(p->peak_min *
                   exp(log(p->peak_max / p->peak_min) * uniform(key, 6 * i + 5)));
  }
  qsort(tmp, s->n_spots, 6 * sizeof(float), cmp_z);
  s->sz = (float *)malloc(s->n_spots * 6 * sizeof(float) + 1);
  if (!s->sz) {
    free(tmp);
    free(s);
    return NULL;
  }
  s->sx = s->sz + s->n_spots;
  s->sy = s->sx + s->n_spots;
  s->sig_xy = s->sy + s->n_spots;
  s->sig_z = s->sig_xy + s->n_spots;
  s->peak = s->sig_z + s->n_spots;
  for (size_t i = 0; i < s->n_spots; i++) {
    s->sz[i] = tmp[6 * i + 0];
    s->sx[i] = tmp[6 * i + 1];
    s->sy[i] = tmp[6 * i + 2];
    s->sig_xy[i] = tmp[6 * i + 3];
    s->sig_z[i] = tmp[6 * i + 4];
    s->peak[i] = tmp[6 * i + 5];
  }
  free(tmp);
  s->sig_z_max = p->sigma_z_max;
  return s;
}

void sf_synth_close(sf_synth *s) {
  if (!s)
    return;
  free(s->sz);
  free(s);
}

size_t sf_synth_n_spots(const sf_synth *s) { return s->n_spots; }

/* EIGER2 tiling: modules of 1028 x 512 separated by 12-column and 38-row
 * gaps (4148 = 4 * 1028 + 3 * 12, 4362 = 8 * 512 + 7 * 38). */
static int eiger_gap(uint32_t y, uint32_t x) {
  return (y % 550u) >= 512u || (x % 1040u) >= 1028u;
}

static double frame_fraction(double f, double z, double sig) {
  /* Share of a Gaussian rocking curve centred at z that falls in [f, f+1). */
  const double k = 0.7071067811865476 / sig;
  return 0.5 * (erf((f + 1.0 - z) * k) - erf((f - z) * k));
}

int sf_synth_frame(const sf_synth *s, int frame, uint32_t *out) {
  if (!s || !out || frame < 0 || frame >= s->p.n_frames)
    return -1;
  const sf_synth_params *p = &s->p;
  const size_t h = p->height, w = p->width, n = h * w;
  float *lambda = (float *)malloc(n * sizeof(float));
  if (!lambda)
    return -3;

  /* Background: linear in radius from bg_centre at the centre to bg_edge at
   * the corner, plus optional diffuse rings. */
  const double cy = 0.5 * (double)h, cx = 0.5 * (double)w;
  const double rmax = sqrt(cx * cx + cy * cy);
#pragma omp parallel for schedule(static)
  for (size_t y = 0; y < h; y++) {
    for (size_t x = 0; x < w; x++) {
      const double dy = (double)y + 0.5 - cy, dx = (double)x + 0.5 - cx;
      const double r = sqrt(dx * dx + dy * dy) / rmax;
      double bg = p->bg_centre + (p->bg_edge - p->bg_centre) * r;
      for (int ring = 0; ring < p->n_rings; ring++) {
        const double rr = (ring + 1.0) / (p->n_rings + 1.0);
        const double d = (r - rr) / 0.01;
        bg += p->ring_amplitude * exp(-0.5 * d * d);
      }
      lambda[y * w + x] = (float)bg;
    }
  }

  /* Spots whose rocking curve reaches this frame. */
  const double zreach = 4.0 * s->sig_z_max + 1.0;
  size_t lo = 0, hi = s->n_spots;
  {
    size_t a = 0, b = s->n_spots;
    while (a < b) {
      size_t m = (a + b) / 2;
      if (s->sz[m] < frame - zreach)
        a = m + 1;
      else
        b = m;
    }
    lo = a;
    a = lo, b = s->n_spots;
    while (a < b) {
      size_t m = (a + b) / 2;
      if (s->sz[m] < frame + 1 + zreach)
        a = m + 1;
      else
        b = m;
    }
    hi = a;
  }
  for (size_t i = lo; i < hi; i++) {
    const double sig = s->sig_xy[i];
    const double best = frame_fraction(floor(s->sz[i]), s->sz[i], s->sig_z[i]);
    const double share =
        frame_fraction((double)frame, s->sz[i], s->sig_z[i]) / fmax(best, 1e-12);
    const double amp = s->peak[i] * share;
    if (amp < 0.05)
      continue;
    const int rad = (int)ceil(3.5 * sig);
    const int x0 = (int)floor(s->sx[i]), y0 = (int)floor(s->sy[i]);
    for (int dy = -rad; dy <= rad; dy++) {
      const int y = y0 + dy;
      if (y < 0 || y >= (int)h)
        continue;
      for (int dx = -rad; dx <= rad; dx++) {
        const int x = x0 + dx;
        if (x < 0 || x >= (int)w)
          continue;
        const double ex = x + 0.5 - s->sx[i], ey = y + 0.5 - s->sy[i];
        lambda[(size_t)y * w + x] +=
            (float)(amp * exp(-(ex * ex + ey * ey) / (2.0 * sig * sig)));
      }
    }
  }

  const uint64_t fkey = mix64(p->seed * 0x9E3779B97F4A7C15ull + (uint64_t)frame);
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < n; k++)
    out[k] = poisson(lambda[k], mix64(fkey ^ (uint64_t)k));
  free(lambda);

  /* Saturated-overload pixels: a valid, large count. */
  if (p->saturated_fraction > 0.0) {
    const uint64_t skey = mix64(fkey ^ 0x5A7ull);
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; k++)
      if (uniform(skey, k) < p->saturated_fraction)
        out[k] = p->saturated_value;
  }

  /* Masks, all written as the masked sentinel. They are fixed across the
   * sweep (a detector's gaps and hot pixels do not move). */
  const uint32_t MASKED = 0xFFFFFFFFu;
  if (p->eiger_gaps) {
#pragma omp parallel for schedule(static)
    for (size_t y = 0; y < h; y++)
      for (size_t x = 0; x < w; x++)
        if (eiger_gap((uint32_t)y, (uint32_t)x))
          out[y * w + x] = MASKED;
  }
  for (uint32_t y = p->row_band_start; y < p->row_band_start + p->row_band_len && y < h; y++)
    for (size_t x = 0; x < w; x++)
      out[y * w + x] = MASKED;
  for (size_t y = 0; y < h; y++)
    for (uint32_t x = p->col_band_start; x < p->col_band_start + p->col_band_len && x < w; x++)
      out[y * w + x] = MASKED;
  const uint64_t hkey = mix64(p->seed ^ 0x407ull);
  for (uint32_t i = 0; i < p->n_hot; i++)
    out[mix64(hkey + i) % n] = MASKED;
  return 0;
}
