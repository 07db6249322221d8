/* Seeded synthetic rotation sweeps (uint32 frames) for tests and benchmarks.
 * See synth.c. */
#ifndef SF_SYNTH_H
#define SF_SYNTH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  uint32_t height, width;
  uint64_t seed;
  int n_frames;
  double bg_edge, bg_centre;  /* Poisson mean at the corner and the centre */
  int n_rings;                /* diffuse rings at evenly spaced radii */
  double ring_amplitude;      /* added mean at the ring's crest */
  double spots_per_frame;     /* mean spots visible on one frame */
  double sigma_xy_min, sigma_xy_max;
  double sigma_z_min, sigma_z_max; /* in frames */
  double peak_min, peak_max;  /* log-uniform peak counts */
  int eiger_gaps;             /* EIGER2 module gaps, masked */
  uint32_t row_band_start, row_band_len; /* a masked band of rows */
  uint32_t col_band_start, col_band_len; /* a masked band of columns */
  uint32_t n_hot;             /* hot pixels, masked */
  double saturated_fraction;  /* pixels set to saturated_value */
  uint32_t saturated_value;
} sf_synth_params;

typedef struct sf_synth sf_synth;

void sf_synth_default_params(sf_synth_params *p);
sf_synth *sf_synth_open(const sf_synth_params *p);
void sf_synth_close(sf_synth *s);
size_t sf_synth_n_spots(const sf_synth *s);
/* Frame `frame` (0-based) of the sweep into out[height * width]. */
int sf_synth_frame(const sf_synth *s, int frame, uint32_t *out);

#ifdef __cplusplus
}
#endif

#endif
