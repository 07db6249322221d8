/*
 * CPU oracle for the spot-finder hot path. TEST INFRASTRUCTURE ONLY: the
 * parity tests, the smoke check and the CPU-baseline leg of the benchmark
 * call this as the checker. Nothing in the product links it.
 *
 * A plain-C restatement of the reference's CPU path:
 *   - or_dext_*   restates dext<T>() (src/spots/dext.cc:9-222), generalised
 *                 to the threshold parameters dials.find_spots exposes. At the
 *                 defaults (dispersion_extended, kernel 3,3, gain 1, sigma_b 6,
 *                 sigma_s 3, min_local 2, global threshold 0) every operation
 *                 and its order is the reference's, so the result is the same
 *                 bit for bit; the tests pin that against fixtures produced by
 *                 the reference itself.
 *   - or_label_*  restates dials_spots::Labeller (src/spots/dials_spots.cc).
 *
 * Build with -ffp-contract=off: the reference is compiled in ISO mode
 * (CMakeLists.txt:8-10), where GCC does not contract a*b+c into an FMA, and an
 * aarch64 GNU-mode build would otherwise change the FP64 decisions.
 */
#ifndef SF_ORACLE_H
#define SF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* src/spots/signal_pixel.hh:20-28 */
typedef struct {
  uint32_t index;
  uint32_t value;
  float background;
  uint16_t population;
  uint16_t reserved;
} or_signal_pixel;

enum { OR_DISPERSION_EXTENDED = 0, OR_DISPERSION = 1 };

typedef struct {
  int algorithm;      /* OR_DISPERSION_EXTENDED (the reference) or OR_DISPERSION */
  int kernel_x;       /* half-width of the local window along x (3: 7 wide) */
  int kernel_y;       /* half-height along y (3) */
  double gain;        /* 1 */
  double sigma_b;     /* 6 */
  double sigma_s;     /* 3 */
  int min_local;      /* 2: windows with fewer valid pixels are not tested */
  double global_threshold; /* 0: a pixel must exceed this to be signal */
} or_params;

void or_default_params(or_params *p);

/*
 * Threshold one frame. Returns 0, or -1 for a bad argument (null image, zero
 * extent, more than INT32_MAX pixels: dext.cc:9-35), or -2 if more than `cap`
 * signal pixels were found (the count is still stored in *found).
 * `mask_out`, if not null, receives one byte per pixel: 1 where signal.
 */
int or_dext_u32(const uint32_t *image, size_t height, size_t width,
                const or_params *params, or_signal_pixel *out, size_t cap,
                size_t *found, uint8_t *mask_out);
int or_dext_u16(const uint16_t *image, size_t height, size_t width,
                const or_params *params, or_signal_pixel *out, size_t cap,
                size_t *found, uint8_t *mask_out);

/* ---- 3-D labelling, src/spots/dials_spots.hh:47-158 ---- */

typedef struct {
  int32_t frame;
  uint32_t index;
  uint32_t value;
} or_pixel;

typedef struct {
  int32_t bbox[6];
  double position[3];
  double variance[3];
  double intensity;
  double intensity_variance;
  uint32_t n_signal;
  uint64_t first;
} or_spot;

typedef struct {
  uint64_t signal_pixels, groups, too_small, too_large, separated, accepted;
} or_counts;

typedef struct or_labeller or_labeller;

/* Returns null on the errors the reference constructor throws for. */
or_labeller *or_label_open(size_t height, size_t width, size_t min_spot_size,
                           size_t max_spot_size, double max_separation,
                           int two_d);
/* 0, or -1 (frame out of order / duplicate), -2 (pixel off the frame or not
 * ascending), -3 (allocation). */
int or_label_add(or_labeller *l, int64_t frame, const or_signal_pixel *signal,
                 size_t n);
void or_label_finish(or_labeller *l);
size_t or_label_n_spots(const or_labeller *l);
size_t or_label_n_pixels(const or_labeller *l);
const or_spot *or_label_spots(const or_labeller *l);
const or_pixel *or_label_pixels(const or_labeller *l);
void or_label_counts(const or_labeller *l, or_counts *out);
void or_label_close(or_labeller *l);

/* Frame decompression (sf_oracle_decompress.c): decompress::image
 * (src/spots/decompress.cc:77-134) with LZ4 blocks and bitshuffle. */
long or_lz4_decode(const uint8_t *in, size_t n, uint8_t *out, size_t cap);
void or_bitunshuffle(const uint8_t *in, uint8_t *out, size_t n, size_t esize);
size_t or_bshuf_default_block(size_t esize);
long or_bshuf_decompress_lz4(const uint8_t *in, size_t n_in, uint8_t *out, size_t size,
                             size_t esize, size_t block_size);
size_t or_frame_bytes(size_t height, size_t width, unsigned bit_depth);
int or_decompress_image(const uint8_t *data, size_t n, const char *algorithm,
                        unsigned bit_depth, size_t height, size_t width, uint8_t *out,
                        size_t out_bytes, char *err, size_t err_cap);

/* Frame scans (sf_oracle_frames.c): mxi_max's scan<T> (apps/mxi_max.cc:47-67)
 * into out = {largest, bad, joins, over}, and find_spots.cc:169-182's
 * narrow_to_16. */
void or_scan_u16(const uint16_t *pixels, size_t n, uint64_t out[4]);
void or_scan_u32(const uint32_t *pixels, size_t n, uint64_t out[4]);
int or_narrow_to_16(const uint32_t *in, size_t n, uint16_t *out, uint32_t *offending);

#ifdef __cplusplus
}
#endif

#endif
