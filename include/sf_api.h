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
#define SF_EBUSY (-5) /* the served form's device-memory budget is taken */
#define SF_EDATA (-6) /* a compressed chunk that does not describe its frame */

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

/*
 * Frame decompression on the device. Replaces decompress::frame_bytes and
 * decompress::image (src/spots/decompress.hh:18-30, decompress.cc:72-134):
 * `data` is a chunk exactly as HDF5 stored it, filter header and all, in host
 * memory (pinned by sf_host_alloc for full speed); `algorithm` is "bslz4"
 * (bitshuffle+LZ4, 16- or 32-bit pixels), "lz4" or "" (uncompressed).
 * Returns 0; -6 (SF_EDATA) where the reference throws, with its text in
 * sf_last_error(); -1 for null pointers; -4 for bitshuffle chunks of other
 * pixel sizes, and for blocks of 4 GB or more decoded (2 GB or more
 * compressed); -3.
 *
 * sf_decompress_image writes the frame to host memory `out`;
 * sf_decompress_device to device memory d_out (16-byte aligned), returning
 * once it is there. out_bytes is the room at out / d_out.
 */
size_t sf_frame_bytes(size_t height, size_t width, unsigned bit_depth);
int sf_decompress_image(const uint8_t *data, size_t nbytes, const char *algorithm,
                        unsigned bit_depth, size_t height, size_t width, uint8_t *out,
                        size_t out_bytes);
int sf_decompress_device(const uint8_t *data, size_t nbytes, const char *algorithm,
                         unsigned bit_depth, size_t height, size_t width, void *d_out,
                         size_t out_bytes);

/*
 * The worker's step of find_spots.cc:772-800 in one call: a compressed chunk
 * (as sf_decompress_image takes it) decoded on the device and thresholded
 * there as sf_find_u16_params / sf_find_u32_params (bit_depth 16 or 32)
 * would threshold the decoded frame. Only the chunk crosses the host link.
 * Returns as sf_find_u32 does, or -6 / -4 as sf_decompress_image.
 */
int sf_find_compressed(const uint8_t *data, size_t nbytes, const char *algorithm,
                       unsigned bit_depth, size_t height, size_t width,
                       const sf_threshold_params *params, sf_signal_pixel *out,
                       size_t capacity, size_t *found);

/*
 * --gpu-force on the device (find_spots.cc:781-795): a 32-bit frame (a chunk
 * as above, or "" with the raw frame) decoded, narrowed to 16 bits as
 * narrow_to_16 does (find_spots.cc:169-182: each value's low 16 bits) and
 * thresholded as a 16-bit frame. *offending receives the largest valid
 * count; at or above 0xFFFD the frame is refused with -6 (SF_EDATA), the
 * reference's "too large for 16 bits" refusal.
 */
int sf_find_narrowed(const uint8_t *data, size_t nbytes, const char *algorithm, size_t height,
                     size_t width, const sf_threshold_params *params, sf_signal_pixel *out,
                     size_t capacity, size_t *found, uint32_t *offending);

/*
 * mxi_max's scan<T> (apps/mxi_max.cc:47-67) on the device: the largest
 * count on a valid pixel (not max() - 1, a bad pixel, nor max(), a tile
 * join), how many pixels are each marker, and how many valid pixels are at
 * 0xFFFD or above. sf_scan_device scans a 16- or 32-bit frame in device
 * memory; sf_scan_compressed is mxi_max's worker step (decompress::image,
 * then scan<T>) with the chunk decoded on the device. Both return when *out
 * is written.
 */
typedef struct {
  uint64_t largest, bad, joins, over;
} sf_frame_scan;
int sf_scan_device(const void *d_image, size_t n_pixels, unsigned bit_depth,
                   sf_frame_scan *out);
int sf_scan_compressed(const uint8_t *data, size_t nbytes, const char *algorithm,
                       unsigned bit_depth, size_t height, size_t width, sf_frame_scan *out);

/* Replaces gpu::profile_stages / gpu::last_stage_times
 * (src/spots/dext_gpu.hh:89-127). Times in milliseconds for the calling
 * thread's last profiled call (host frame, device frame or batch, all its
 * frames): upload (host-frame calls), `fused` (the whole threshold), copy
 * (list read-back). On the 32-bit dispersion_extended path also stage0
 * (stage 0 and the erosion, one kernel: the reference's stage0 + stage1),
 * stage2 and sort (ordering the list); stage1 stays 0. A device call's
 * times are read when sf_last_stage_times is called, which waits for it. */
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
 *                capacity, in which case the list is incomplete); 0xFFFFFFFE
 *                if a bounded device wait of the launch ran out (no list;
 *                the host-frame calls return -3 for it)
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
 * Batched device threshold (no reference counterpart; the reference's -j
 * workers run one frame per call, src/apps/find_spots.cc:760-833): up to
 * SF_MAX_BATCH same-shaped frames in one launch sequence, with the results
 * of each frame equal to a single-frame call on it.
 *   d_images     host array of n_frames device pointers (16-byte aligned
 *                frames read as 128-bit rows; others work, slower)
 *   d_out        n_frames * capacity records: frame j's list at j * capacity
 *   d_bits       n_frames * ceil(width/32) * height words, frame after frame
 *   d_counts     n_frames uint32 counts
 *   d_word_prefix optional (NULL): n_frames * the words of one mask
 *   d_workspace  sf_batch_workspace_bytes(n_frames, height, width, capacity)
 * sf_batch_workspace_bytes returns 0 for a shape or batch size it refuses.
 */
#define SF_MAX_BATCH 64
size_t sf_batch_workspace_bytes(size_t n_frames, size_t height, size_t width,
                                size_t capacity);
int sf_threshold_u32_batch_device(const uint32_t *const *d_images, size_t n_frames,
                                  size_t height, size_t width,
                                  const sf_threshold_params *params, sf_signal_pixel *d_out,
                                  size_t capacity, uint32_t *d_bits, uint32_t *d_counts,
                                  uint32_t *d_word_prefix, void *d_workspace,
                                  size_t workspace_bytes, void *stream);
int sf_threshold_u16_batch_device(const uint16_t *const *d_images, size_t n_frames,
                                  size_t height, size_t width,
                                  const sf_threshold_params *params, sf_signal_pixel *d_out,
                                  size_t capacity, uint32_t *d_bits, uint32_t *d_counts,
                                  uint32_t *d_word_prefix, void *d_workspace,
                                  size_t workspace_bytes, void *stream);

/*
 * Batches of frames of different shapes (detectors of different sizes; no
 * reference counterpart: the reference thresholds one frame a call,
 * src/spots/dext_cuda.cu:711-869). Frame j is heights[j] x widths[j]; every
 * output is laid out for the batch's envelope H x W (the largest height and
 * the largest width): frame j's list at d_out + j * capacity, its count at
 * d_counts[j], its mask at d_bits + j * sf_mixed_batch_mask_words(...) (=
 * ceil(W/32) * H words) in its own rows of ceil(widths[j]/32) words, the
 * optional word positions likewise. For 32-bit frames with the reference's
 * window (kernel 3,3, dispersion_extended, gain 1, integral sigmas) the
 * whole batch is one launch sequence; other settings run frames of another
 * shape one launch sequence each. The workspace is
 * sf_mixed_batch_workspace_bytes (the batch workspace of the envelope).
 */
size_t sf_mixed_batch_workspace_bytes(size_t n_frames, const size_t *heights,
                                      const size_t *widths, size_t capacity);
size_t sf_mixed_batch_mask_words(size_t n_frames, const size_t *heights, const size_t *widths);
int sf_threshold_u32_mixed_batch_device(const uint32_t *const *d_images, const size_t *heights,
                                        const size_t *widths, size_t n_frames,
                                        const sf_threshold_params *params,
                                        sf_signal_pixel *d_out, size_t capacity,
                                        uint32_t *d_bits, uint32_t *d_counts,
                                        uint32_t *d_word_prefix, void *d_workspace,
                                        size_t workspace_bytes, void *stream);

/*
 * Batch plans (no reference counterpart): one frame shape with its device
 * outputs and workspace. sf_plan_run enqueues the batched threshold of
 * n_frames <= max_frames device frames (as sf_threshold_u32_batch_device);
 * after the first run the launch sequence is captured as a CUDA graph and
 * replayed whenever the same frame pointers come again (up to 16 pointer
 * sets are kept). sf_plan_tune times, on the given frames, the frames a
 * launch sequence takes (all, 32 or 16; sf_plan_frames_per_launch, 0 for
 * all) and the strip run lengths (sf_plan_run_rows), and keeps the fastest
 * pair; the results are the same for any of them. Outputs (device pointers, valid until sf_plan_destroy): frame j's
 * list at sf_plan_lists(p) + j * capacity, its count at sf_plan_counts(p)[j],
 * its mask at sf_plan_masks(p) + j * ceil(width/32) * height. NULL on failure
 * (the reason in sf_last_error()).
 */
typedef struct sf_plan sf_plan;
sf_plan *sf_plan_create(size_t height, size_t width, size_t max_frames, size_t capacity,
                        const sf_threshold_params *params);
void sf_plan_destroy(sf_plan *plan);
int sf_plan_run(sf_plan *plan, const uint32_t *const *d_images, size_t n_frames, void *stream);
int sf_plan_tune(sf_plan *plan, const uint32_t *const *d_images, size_t n_frames, void *stream);
int sf_plan_run_rows(const sf_plan *plan);
size_t sf_plan_frames_per_launch(const sf_plan *plan);
/* Sets what sf_plan_tune would choose (a run length, 0 for the default
 * geometry; frames a launch sequence, 0 for all), e.g. from an earlier
 * tuning of the same detector; drops the plan's graphs. */
int sf_plan_configure(sf_plan *plan, int run_rows, size_t frames_per_launch);
size_t sf_plan_graphs(const sf_plan *plan);
sf_signal_pixel *sf_plan_lists(const sf_plan *plan);
uint32_t *sf_plan_counts(const sf_plan *plan);
uint32_t *sf_plan_masks(const sf_plan *plan);
/* Waits for the plan's work and copies frame j's list to the host: 0, or -2
 * with *found the count when it exceeds the plan's or this capacity. */
int sf_plan_result(sf_plan *plan, size_t j, sf_signal_pixel *out, size_t capacity,
                   size_t *found);

/* ---- 3-D spot labelling (src/spots/dials_spots.hh) ---- */

/* dials_spots::Pixel (src/spots/dials_spots.hh:50-54): a signal pixel of an
 * accepted spot, kept for the shoebox. */
typedef struct {
  int32_t frame;
  uint32_t index;
  uint32_t value;
} sf_pixel;

/* dials_spots::Spot (src/spots/dials_spots.hh:57-79), same layout. */
typedef struct {
  int32_t bbox[6];            /* x0, x1, y0, y1, z0, z1; upper bounds exclusive */
  double position[3];         /* xyzobs.px.value */
  double variance[3];         /* xyzobs.px.variance */
  double intensity;           /* intensity.sum.value */
  double intensity_variance;  /* intensity.sum.variance */
  uint32_t n_signal;
  uint64_t first;             /* where its pixels start in the pixel list */
} sf_spot;

/* dials_spots::Options (src/spots/dials_spots.hh:81-95). */
typedef struct {
  size_t min_spot_size;   /* 3 */
  size_t max_spot_size;   /* 1000 */
  double max_separation;  /* 2.0; <= 0 turns the filter off */
  int two_d;              /* 0 */
} sf_label_options;

/* dials_spots::Counts (src/spots/dials_spots.hh:99-106). */
typedef struct {
  uint64_t signal_pixels, groups, too_small, too_large, separated, accepted;
} sf_counts;

typedef struct sf_labeller sf_labeller;

void sf_default_label_options(sf_label_options *options);

/* Replaces dials_spots::Labeller::Labeller (src/spots/dials_spots.hh:110,
 * dials_spots.cc:21-30): NULL, with the reason in sf_last_error(), on the
 * errors the constructor throws for. live_capacity bounds the pixels held
 * open at once plus one batch's (0: 4 Mi); exceeding it is reported by the
 * add as -2. The labeller's device state is resident until sf_label_close. */
sf_labeller *sf_label_open(size_t height, size_t width,
                           const sf_label_options *options,
                           size_t live_capacity);
void sf_label_close(sf_labeller *labeller);

/* Replaces Labeller::add (src/spots/dials_spots.hh:114,
 * dials_spots.cc:57-145) for one frame's host list, ascending by index.
 * -1 if the frame is out of order or the list is off the frame or not
 * ascending (the reference throws there). */
int sf_label_add(sf_labeller *labeller, int64_t frame,
                 const sf_signal_pixel *signal, size_t n);

/* Labeller::add for n_frames ascending frames at once, their lists already
 * on the device (frame j's at d_lists + j * list_stride, its count in
 * d_counts[j]), e.g. straight from sf_threshold_*_device; enqueued on
 * `stream`, the stream that produced the lists (NULL: the legacy default
 * stream), which is synchronised before the call returns. At most 64 frames
 * per call. No reference counterpart: the reference adds one host list at a
 * time. */
int sf_label_add_device(sf_labeller *labeller, const int64_t *frames,
                        size_t n_frames, const sf_signal_pixel *d_lists,
                        size_t list_stride, const uint32_t *d_counts,
                        void *stream);

/* Replaces Labeller::finish (src/spots/dials_spots.hh:117). */
int sf_label_finish(sf_labeller *labeller);

/* Replace Labeller::spots(), pixels(), counts(), live()
 * (src/spots/dials_spots.hh:119-125). The spots and kept pixels are held in
 * device memory as they are produced; sf_label_spots / sf_label_pixels copy
 * them to the caller's buffer (waiting for the last add), and return -2 if
 * capacity is short. */
size_t sf_label_n_spots(const sf_labeller *labeller);
size_t sf_label_n_pixels(const sf_labeller *labeller);
int sf_label_spots(const sf_labeller *labeller, sf_spot *out, size_t capacity);
int sf_label_pixels(const sf_labeller *labeller, sf_pixel *out,
                    size_t capacity);
void sf_label_counts(const sf_labeller *labeller, sf_counts *out);
size_t sf_label_live(const sf_labeller *labeller);

/* ---- The reflection table (src/spots/refl.hh) ---- */

/* refl::Options (src/spots/refl.hh:53-64). identifier NULL or "" writes an
 * empty identifier map. */
typedef struct {
  size_t panel;            /* 0 */
  int id;                  /* 0 */
  const char *identifier;  /* NULL */
  int shoeboxes;           /* 1 */
} sf_refl_options;

void sf_default_refl_options(sf_refl_options *options);

/* Replaces refl::write (src/spots/refl.hh:72-74, refl.cc:223-351): the DIALS
 * .refl of spots (with their kept pixels, for the shoeboxes) in host memory,
 * byte for byte the reference's file. Needs no GPU. -1 for no path, a zero
 * width, spots whose pixels or boxes are not in the arrays, or a file that
 * cannot be written (reason in sf_last_error()); -4 when the shoebox column
 * would exceed msgpack's 4 GB binary (the reference throws for both). */
int sf_refl_write(const char *path, const sf_spot *spots, size_t n_spots,
                  const sf_pixel *pixels, size_t n_pixels, size_t width,
                  const sf_refl_options *options);

/* refl::write of a device labeller's spots: the same file as sf_refl_write
 * on sf_label_spots / sf_label_pixels, with the shoebox column built in
 * device memory from the labeller's device-resident pixels and copied out
 * once (after the labeller's last add). No reference counterpart as an entry
 * point: the reference writes from host vectors. -3 on a CUDA failure. */
int sf_label_write_refl(const sf_labeller *labeller, const char *path,
                        const sf_refl_options *options);

/*
 * sf_threshold_u32_device as above, for callers that cannot allocate device
 * memory: a plugin inside a host application whose own allocator owns all
 * device memory, or a detector-stream loop that must not stall on an
 * allocation. It has no counterpart in the reference. Its scratch is a fixed
 * 32 MiB array inside this library, so it takes no workspace and calls no
 * allocator; the caller still passes the frame and every output.
 *   - A call needs the workspace layout of (height, width, capacity), i.e.
 *     sf_workspace_bytes(height, width, capacity), to fit in the 32 MiB, and
 *     capacity at most 524288 records; otherwise it returns -1 with the
 *     reason in sf_last_error(). Both hold for an EIGER2 16M frame
 *     (4362 x 4148) at the full 524288 records, and for any frame of up to
 *     2^25 pixels whose sides are both at least 256.
 *   - The driver reserves the 32 MiB on a device when this library's module
 *     holding the array is first loaded there (with CUDA's lazy module
 *     loading, at the first use of that module on the device, which may
 *     synchronise), and keeps it until the process exits. The first call on
 *     each device also looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current. So make one warm-up
 *     call on each device before acquisition starts and before any stream
 *     capture.
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

/*
 * The served form (no reference counterpart; the reference's mxi_find reads
 * one sweep from disk): a request loop for frames arriving from several
 * detector streams at once. Each open sweep keeps its frame ring and its 3-D
 * labeller resident on the device; sweeps are admitted against a device
 * memory budget (sf_server_open_sweep returns SF_EBUSY when it is taken:
 * retry once another sweep closes). Frames are submitted in ascending order
 * per sweep from host memory (page-locked, e.g. sf_host_alloc, for a fast
 * copy) that must stay untouched until the frame is reported done. A worker
 * thread copies them in, thresholds whatever is ready across sweeps of one
 * shape and parameter set in one launch (up to max_batch frames) and labels
 * each sweep's frames in order; sf_server_poll returns the finished frames
 * with their submit-to-labelled latency. After sf_server_finish_sweep the
 * sweep's spots are read from its labeller (sf_server_labeller, sf_label_*).
 * A frame's results do not depend on the other sweeps in the mix.
 */
typedef struct {
  size_t hbm_budget;       /* device bytes for sweeps and the spots and pixels they
                              hold on the device; 0: 80% of the free memory. A
                              sweep whose results would take the server past it
                              fails with -5 (SF_EBUSY) instead of growing */
  size_t max_batch;        /* frames per threshold launch, 1..SF_MAX_BATCH (16) */
  size_t ring;             /* device frame slots per sweep, >= max_batch (32) */
  size_t capacity_divisor; /* signal-list capacity = pixels / this (16) */
  size_t coalesce_us;      /* wait up to this long to fill a launch or a label call (1000) */
  size_t label_capacity;   /* live pixels each sweep's labeller holds: its open
                              components plus one label call's frames (0: min(4 Mi,
                              pixels / 2); dense frames need more) */
} sf_server_options;

typedef struct {
  int64_t sweep, frame;
  uint32_t n_signal;       /* signal pixels of the frame */
  int status;              /* 0, or the error code of its sweep */
  double latency_ms;       /* from sf_server_submit to labelled */
} sf_frame_done;

/* Counters since sf_server_open: threshold launches and the frames in them,
 * label calls and their frames, host seconds spent launching batches and in
 * label calls (summed over the sweeps' labellers), and the longest single
 * launch and label call. */
typedef struct {
  uint64_t batches, batch_frames, label_calls, label_frames;
  double launch_seconds, label_seconds;
  double launch_max_seconds, label_max_seconds;
} sf_server_stats;

typedef struct sf_server sf_server;
void sf_default_server_options(sf_server_options *options);
sf_server *sf_server_open(const sf_server_options *options);
void sf_server_close(sf_server *server);
size_t sf_server_sweep_bytes(const sf_server *server, size_t height, size_t width,
                             const sf_label_options *label);
size_t sf_server_used_bytes(const sf_server *server);
void sf_server_get_stats(sf_server *server, sf_server_stats *out);
int sf_server_open_sweep(sf_server *server, size_t height, size_t width,
                         const sf_threshold_params *params, const sf_label_options *label,
                         int64_t *sweep);
int sf_server_submit(sf_server *server, int64_t sweep, int64_t frame,
                     const uint32_t *host_frame);
/* As sf_server_submit for a frame stored as a compressed chunk (the input of
 * decompress::image, src/spots/decompress.hh:28-30: "bslz4", "lz4", or ""
 * for raw 32-bit pixels). The chunk's header and framing are checked here:
 * -6 (SF_EDATA) with the reference's text, and the frame is not taken. The
 * chunk (pinned host memory, kept until the frame is done) is copied to the
 * device and decoded into the sweep's slot; a block the decoder refuses fails
 * its frame and the sweep with SF_EDATA. */
int sf_server_submit_chunk(sf_server *server, int64_t sweep, int64_t frame,
                           const uint8_t *data, size_t nbytes, const char *algorithm);
/* Up to max finished frames; waits up to wait_ms for the first one. */
size_t sf_server_poll(sf_server *server, sf_frame_done *out, size_t max, int wait_ms);
int sf_server_finish_sweep(sf_server *server, int64_t sweep);
sf_labeller *sf_server_labeller(sf_server *server, int64_t sweep);
/* The message of a sweep's first failure ("" if none). */
const char *sf_server_sweep_error(sf_server *server, int64_t sweep);
int sf_server_close_sweep(sf_server *server, int64_t sweep);

#ifdef __cplusplus
}
#endif

#endif /* SF_API_H */
