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

/* Compressed chunks as an HDF5 writer stores them (synth_chunk.c): the
 * 12-byte filter header and bitshuffle+LZ4 ("bslz4") or LZ4 ("lz4") blocks.
 * block_bytes 0 takes bitshuffle's default block (bslz4) or one block for the
 * frame (lz4). Each returns the chunk's length, or -1 (bad arguments, or
 * more than cap bytes). */
size_t sf_chunk_bound(size_t frame_bytes, size_t block_bytes);
int64_t sf_chunk_bslz4(const void *frame, size_t n_elems, unsigned esize, size_t block_bytes,
                       uint8_t *out, size_t cap);
int64_t sf_chunk_lz4(const void *frame, size_t nbytes, size_t block_bytes, uint8_t *out,
                     size_t cap);
/* One LZ4 block of n bytes into dst (sf_lz4_bound(n) bytes); its length. */
size_t sf_lz4_bound(size_t n);
size_t sf_lz4_block(const uint8_t *src, size_t n, uint8_t *dst);
/* The bit planes of n elements (n a multiple of 8) of esize bytes. */
void sf_bitshuffle(const uint8_t *in, uint8_t *out, size_t n, size_t esize);

#ifdef __cplusplus
}
#endif

#endif
