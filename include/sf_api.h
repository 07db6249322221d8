/*
 * sf_api.h -- the C ABI of the GB300 spot finder (libsfgb.so).
 *
 * This is the drop-in boundary for the spot-finder hot path of dials-metal:
 * the threshold backend behind `namespace gpu` in src/spots/dext_gpu.hh, and
 * the 3-D labelling of src/spots/dials_spots.hh. Plain pointers and sizes
 * only. Each entry point names the reference interface it replaces.
 *
 * Return codes follow the reference (src/spots/dext_gpu.hh:156-170,
 * src/spots/dext.cc:14-23): 0 success, -1 bad argument, -2 more signal than
 * the output holds. -3 is a CUDA failure (the reference throws
 * std::runtime_error("CUDA: ...") there, src/spots/dext_cuda.cu:46-51); the
 * message is in sf_last_error(). -4 is "this backend cannot do that" (the
 * reference's runtime_error for an unsupported pixel type).
 *
 * Threading: every host entry point may be called from several threads at
 * once; each thread gets its own stream and device buffers, as the
 * reference's per-thread Workspace (src/spots/dext_cuda.cu:471-545).
 */
#ifndef SF_API_H
#define SF_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SF_OK 0
#define SF_EBADARG (-1)
#define SF_EOVERFLOW (-2)
#define SF_ECUDA (-3)
#define SF_EUNSUPPORTED (-4)

/* src/spots/signal_pixel.hh:20-28: one surviving pixel, 16 bytes. */
typedef struct {
  uint32_t index;      /* row-major position in the frame */
  uint32_t value;      /* the raw pixel */
  float background;    /* the masked local mean at that pixel */
  uint16_t population; /* pixels that mean was averaged over */
  uint16_t reserved;   /* 0 */
} sf_signal_pixel;

enum { SF_DISPERSION_EXTENDED = 0, SF_DISPERSION = 1 };

/* Threshold parameters. The reference hard-wires the defaults
 * (src/spots/dext.cc:37-40, :99, :203); sf_default_params() returns them.
 * Kernel sizes are square, half-width 2, 3 or 4. */
typedef struct {
  int algorithm;           /* SF_DISPERSION_EXTENDED (reference) | SF_DISPERSION */
  int kernel_x, kernel_y;  /* 3, 3 */
  double gain;             /* 1 */
  double sigma_b;          /* 6 */
  double sigma_s;          /* 3 */
  int min_local;           /* 2 */
  double global_threshold; /* 0 */
} sf_threshold_params;

void sf_default_params(sf_threshold_params *params);

/* Replaces gpu::backend() (src/spots/dext_gpu.hh:29). */
const char *sf_backend(void);

/* Replaces gpu::available() / gpu::unavailable_reason()
 * (src/spots/dext_gpu.hh:137-141). */
int sf_available(void);
const char *sf_unavailable_reason(void);

/* Replaces gpu::memory_free() (src/spots/dext_gpu.hh:146). */
size_t sf_memory_free(void);

/* Replace gpu::host_alloc / gpu::host_free (src/spots/dext_gpu.hh:153-154):
 * page-locked memory, or NULL on failure. */
void *sf_host_alloc(size_t bytes);
void sf_host_free(void *pointer);

/* The last error message on the calling thread ("" if none). */
const char *sf_last_error(void);

/*
 * Replaces gpu::find<std::uint32_t> / gpu::find<std::uint16_t>
 * (src/spots/dext_gpu.hh:156-180; src/spots/dext_cuda.cu:711-869): threshold
 * one host frame, height x width row-major, into `out` (room for `capacity`
 * records), ascending by index, `*found` records. Returns 0, -1, -2 (then
 * *found is the count that did not fit), -3.
 */
int sf_find_u32(const uint32_t *image, size_t height, size_t width,
                sf_signal_pixel *out, size_t capacity, size_t *found);
int sf_find_u16(const uint16_t *image, size_t height, size_t width,
                sf_signal_pixel *out, size_t capacity, size_t *found);

/* As sf_find_u32/u16 with explicit threshold parameters (NULL: defaults).
 * No reference counterpart: the reference hard-wires them (dext.cc:37-40). */
int sf_find_u32_params(const uint32_t *image, size_t height, size_t width,
                       const sf_threshold_params *params, sf_signal_pixel *out,
                       size_t capacity, size_t *found);
int sf_find_u16_params(const uint16_t *image, size_t height, size_t width,
                       const sf_threshold_params *params, sf_signal_pixel *out,
                       size_t capacity, size_t *found);

/* Replaces gpu::profile_stages / gpu::last_stage_times
 * (src/spots/dext_gpu.hh:89-127). Times in milliseconds for the calling
 * thread's last profiled frame: upload, the fused threshold (reported as
 * `fused`), copy (list read-back). stage0/1/2 and sort stay 0: the stages
 * run as one kernel and the list arrives sorted. */
typedef struct {
  double upload, stage0, stage1, stage2, fused, copy, sort;
} sf_stage_times;
void sf_profile_stages(int on);
int sf_profiling(void);
void sf_last_stage_times(sf_stage_times *out);

/*
 * Device-resident threshold (no reference counterpart: the reference always
 * starts from a host frame). All pointers are device pointers; `stream` is a
 * cudaStream_t (NULL: the legacy default stream). Enqueues the work and
 * returns without synchronising.
 *   d_image      height x width pixels
 *   d_out        room for `capacity` records; filled ascending by index
 *   d_bits       ceil(width/32) * height words: the strong-pixel bitmask
 *   d_count      one uint32: the number of signal pixels found (may exceed
 *                capacity, in which case the list is incomplete)
 *   d_word_prefix optional (NULL): per bitmask word, the list position of
 *                its first pixel
 *   d_workspace  sf_workspace_bytes(height, width, capacity) bytes
 */
size_t sf_workspace_bytes(size_t height, size_t width, size_t capacity);
int sf_threshold_u32_device(const uint32_t *d_image, size_t height,
                            size_t width, const sf_threshold_params *params,
                            sf_signal_pixel *d_out, size_t capacity,
                            uint32_t *d_bits, uint32_t *d_count,
                            uint32_t *d_word_prefix, void *d_workspace,
                            size_t workspace_bytes, void *stream);
int sf_threshold_u16_device(const uint16_t *d_image, size_t height,
                            size_t width, const sf_threshold_params *params,
                            sf_signal_pixel *d_out, size_t capacity,
                            uint32_t *d_bits, uint32_t *d_count,
                            uint32_t *d_word_prefix, void *d_workspace,
                            size_t workspace_bytes, void *stream);

/*
 * sf_threshold_u32_device as above, for callers that cannot allocate device
 * memory: a plugin inside a host application whose own allocator owns all
 * device memory, or a detector-stream loop that must not stall on an
 * allocation. It has no counterpart in the reference. Its scratch is a fixed
 * 9 MiB array inside this library (held on every GPU that loads the library
 * until exit), so it takes no workspace and calls no allocator; the caller
 * still passes the frame and every output.
 *   - capacity may be at most 524288 records; larger capacities, or frames
 *     whose per-tile bookkeeping would not fit, return -1 with the reason in
 *     sf_last_error().
 *   - The first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture.
 *   - Every call shares the one array: calls whose work overlaps on the GPU
 *     (different streams, or different host threads) race and corrupt each
 *     other's results. Serialise them, e.g. on one stream.
 */
int sf_threshold_u32_device_noalloc(const uint32_t *d_image, size_t height,
                                    size_t width,
                                    const sf_threshold_params *params,
                                    sf_signal_pixel *d_out, size_t capacity,
                                    uint32_t *d_bits, uint32_t *d_count,
                                    uint32_t *d_word_prefix, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SF_API_H */
