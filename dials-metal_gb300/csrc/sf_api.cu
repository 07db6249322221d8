// The C ABI (include/sf_api.h): device discovery, pinned host memory, and
// the per-thread host-frame threshold that replaces gpu::find<T>
// (src/spots/dext_cuda.cu:711-869), plus the device-resident entry points.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "sf_api.h"
#include "sf_common.cuh"
#include "sf_decompress.cuh"
#include "sf_frames.cuh"
#include "sf_scan.cuh"
#include "sf_stream.cuh"
#include "sf_threshold.cuh"

namespace sf {

thread_local std::string t_last_error;
static bool g_profiling = false;
thread_local sf_stage_times t_stage_times = {0, 0, 0, 0, 0, 0, 0};

// Events around the kernel groups of the calling thread's last profiled
// launch; read (after they complete) by sf_last_stage_times.
struct DeviceMarks {
  StreamMarks m = {nullptr, nullptr, nullptr, nullptr};
  bool pending = false, staged = false;
  ~DeviceMarks() {
    for (cudaEvent_t e : {m.start, m.stage01, m.stage2, m.order})
      if (e)
        cudaEventDestroy(e);
  }
  const StreamMarks *arm() {
    if (!m.start)
      for (cudaEvent_t *e : {&m.start, &m.stage01, &m.stage2, &m.order})
        cudaEventCreate(e);
    pending = true;
    return &m;
  }
  // Moves the device stage times of the last launch into *t (zeros where a
  // launch recorded no stage boundaries).
  void collect(sf_stage_times *t) {
    if (!pending)
      return;
    pending = false;
    if (cudaEventSynchronize(m.order) != cudaSuccess)
      return;
    float ms = 0.0f;
    t->stage0 = t->stage1 = t->stage2 = t->sort = 0.0;
    if (staged) {
      cudaEventElapsedTime(&ms, m.start, m.stage01);
      t->stage0 = ms;
      cudaEventElapsedTime(&ms, m.stage01, m.stage2);
      t->stage2 = ms;
      cudaEventElapsedTime(&ms, m.stage2, m.order);
      t->sort = ms;
    }
    cudaEventElapsedTime(&ms, m.start, m.order);
    t->fused = ms;
  }
};
thread_local DeviceMarks t_marks;
// Set while a plan captures its launch sequence into a graph: no profiling
// events are recorded into it.
thread_local bool t_capturing = false;

int fail(cudaError_t e, const char *what) {
  t_last_error = std::string("CUDA: ") + what + ": " + cudaGetErrorString(e);
  return SF_ECUDA;
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Validates the parameters and precomputes the per-launch constants.
int make_launch_params(const sf_threshold_params *in, LaunchParams *P) {
  sf_threshold_params p;
  if (in)
    p = *in;
  else
    sf_default_params(&p);
  if (p.algorithm != SF_DISPERSION_EXTENDED && p.algorithm != SF_DISPERSION)
    return SF_EBADARG;
  if (p.kernel_x != p.kernel_y || p.kernel_x < 2 || p.kernel_x > kMaxHalf)
    return SF_EUNSUPPORTED;
  if (p.min_local < 0 || !std::isfinite(p.gain) || !std::isfinite(p.sigma_b) ||
      !std::isfinite(p.sigma_s))
    return SF_EBADARG;
  std::memset(P, 0, sizeof(*P));
  P->algorithm = p.algorithm;
  P->half = p.kernel_x;
  P->gain = p.gain;
  P->sigma_b = p.sigma_b;
  P->sigma_s = p.sigma_s;
  P->min_local = (uint32_t)p.min_local;
  // value > global_threshold, as the smallest integer value that passes.
  const double gt = p.global_threshold;
  if (std::isnan(gt))
    P->p_min = ~0ull;
  else if (gt < 0.0)
    P->p_min = 0;
  else if (gt >= 4294967296.0)
    P->p_min = ~0ull;
  else
    P->p_min = (uint64_t)std::floor(gt) + 1ull;
  P->int_ok = p.gain == 1.0 && p.sigma_b == std::floor(p.sigma_b) &&
              p.sigma_b >= 0.0 && p.sigma_b <= 1024.0 &&
              p.sigma_s == std::floor(p.sigma_s) && p.sigma_s >= 0.0 &&
              p.sigma_s <= 1024.0;
  P->sigma_b_int = P->int_ok ? (uint32_t)p.sigma_b : 0;
  P->sigma_s2_int = P->int_ok ? (uint32_t)(p.sigma_s * p.sigma_s) : 0;
  for (int n = 0; n <= kMaxN0; n++) {
    // The reference's sqrt(R(2) * (m - R(1))), correctly rounded on both
    // sides of the bus.
    const double r = std::sqrt(2.0 * ((double)n - 1.0));
    P->root[n] = r;
    P->rootf[n] = std::sqrt(2.0f * ((float)n - 1.0f));
    if (n >= 1) {
      const double scaled = std::ldexp(r, kRootShift); // exact
      P->root_lo[n] = (uint32_t)std::floor(scaled);
      P->root_hi[n] = (uint32_t)std::ceil(scaled);
    }
  }
  return SF_OK;
}

// One workspace serves both threshold paths: the streaming path (32-bit
// frames, dispersion_extended, gain 1 and integral sigmas; one frame or a
// batch) and the tile path (everything else, one frame at a time).
struct WorkspaceLayout {
  size_t staging, cand, res, scr1, amb, wide, counters, block_sums, tile_base, row_total, total;
  size_t cand_cap, words;
};

static WorkspaceLayout layout(size_t h, size_t w, size_t capacity, size_t nframes = 1) {
  WorkspaceLayout L;
  L.words = (w + 31) / 32 * h;
  // A frame with more eroded-mask candidates than twice the list capacity
  // (plus slack) is not a frame of spots; it is refused like an overflow.
  L.cand_cap = std::min(h * w, 2 * capacity + 65536);
  size_t off = 0;
  auto take = [&off](size_t bytes) {
    const size_t at = off;
    off += align_up(bytes ? bytes : 1, 256);
    return at;
  };
  L.staging = take(capacity * sizeof(sf_signal_pixel));  // the tile path's, one frame
  L.cand = take(nframes * L.cand_cap * sizeof(uint32_t));
  L.res = take(nframes * L.cand_cap * sizeof(uint2));
  L.scr1 = take(nframes * L.words * sizeof(uint32_t));
  L.amb = take(nframes * (L.words + 2 * lattice_tiles((int)h, (int)w)) * sizeof(uint32_t));
  L.wide = take(stream_wide_entries((int)h, (int)w, (int)nframes) * 2 * sizeof(uint4));
  L.counters = take(counter_words((int)nframes) * sizeof(uint32_t));
  L.block_sums = take((size_t)std::max(kScanBlocks, stream_order_blocks()) * sizeof(uint32_t));
  L.tile_base = take((size_t)tiles_x((int)w) * tiles_y((int)h) * sizeof(uint32_t));
  L.row_total = take((size_t)tiles_y((int)h) * sizeof(uint32_t));
  L.total = off;
  return L;
}

static bool shape_ok(size_t h, size_t w) {
  // The kernels index in 32 bits, as the reference (dext.cc:17-23).
  return h > 0 && w > 0 && h <= 0x7fffffffu / w;
}

static bool stream_path(size_t elem, const LaunchParams &P) {
  return elem == 4 && P.algorithm == SF_DISPERSION_EXTENDED && P.int_ok;
}

// 16-bit frames take the lattice path for kernel 3,3 (any gain and sigmas:
// their tests are the reference's float ones) when whole 8-byte pieces of 4
// pixels tile every row: 4 | width and 8-byte aligned frames.
template <typename T>
static bool stream16_path(const T *const *d_images, size_t n, const size_t *widths,
                          const LaunchParams &P) {
  if (sizeof(T) != 2 || P.algorithm != SF_DISPERSION_EXTENDED || P.half != 3)
    return false;
  for (size_t j = 0; j < n; j++)
    if (widths[j] % 4 != 0 || reinterpret_cast<uintptr_t>(d_images[j]) % 8 != 0)
      return false;
  return true;
}

// The batch's envelope: its tallest and widest frame (each checked).
static bool envelope(size_t n, const size_t *heights, const size_t *widths, size_t *h,
                     size_t *w) {
  *h = *w = 0;
  for (size_t j = 0; j < n; j++) {
    if (!shape_ok(heights[j], widths[j]))
      return false;
    *h = std::max(*h, heights[j]);
    *w = std::max(*w, widths[j]);
  }
  return n > 0 && shape_ok(*h, *w);
}

template <typename T>
static int threshold_frames_mixed(const T *const *d_images, size_t n, const size_t *heights,
                                  const size_t *widths, const sf_threshold_params *params,
                                  sf_signal_pixel *d_out, size_t capacity, uint32_t *d_bits,
                                  uint32_t *d_counts, uint32_t *d_word_prefix, void *d_ws,
                                  size_t ws_bytes, int run_rows, cudaStream_t stream);

// Frames d_images[0 .. n) (device pointers), all h x w: lists at
// d_out + j * capacity, masks at d_bits + j * words, counts at d_counts[j].
template <typename T>
static int threshold_frames(const T *const *d_images, size_t n, size_t h, size_t w,
                            const sf_threshold_params *params, sf_signal_pixel *d_out,
                            size_t capacity, uint32_t *d_bits, uint32_t *d_counts,
                            uint32_t *d_word_prefix, void *d_ws, size_t ws_bytes,
                            int run_rows, cudaStream_t stream) {
  if (n == 0 || n > (size_t)kMaxBatch)
    return SF_EBADARG;
  size_t hs[kMaxBatch], wsz[kMaxBatch];
  for (size_t j = 0; j < n; j++)
    hs[j] = h, wsz[j] = w;
  return threshold_frames_mixed<T>(d_images, n, hs, wsz, params, d_out, capacity, d_bits,
                                   d_counts, d_word_prefix, d_ws, ws_bytes, run_rows, stream);
}

// Frames d_images[0 .. n) of shapes heights[j] x widths[j], laid out for the
// envelope H x W (the tallest and the widest): lists at d_out + j * capacity,
// frame j's mask at d_bits + j * ceil(W / 32) * H in its own rows of
// ceil(widths[j] / 32) words, counts at d_counts[j]. The kernel-3,3 lattice
// path takes the mixed frames in one launch sequence; other settings run
// frames of another shape one launch sequence each.
template <typename T>
static int threshold_frames_mixed(const T *const *d_images, size_t n, const size_t *heights,
                                  const size_t *widths, const sf_threshold_params *params,
                                  sf_signal_pixel *d_out, size_t capacity, uint32_t *d_bits,
                                  uint32_t *d_counts, uint32_t *d_word_prefix, void *d_ws,
                                  size_t ws_bytes, int run_rows, cudaStream_t stream) {
  size_t h = 0, w = 0;
  if (!d_images || !heights || !widths || n == 0 || n > (size_t)kMaxBatch || !d_out ||
      !d_bits || !d_counts || !d_ws || capacity > 0xffffffffu ||
      !envelope(n, heights, widths, &h, &w))
    return SF_EBADARG;
  bool mixed = false;
  for (size_t j = 0; j < n; j++) {
    if (!d_images[j])
      return SF_EBADARG;
    mixed |= heights[j] != h || widths[j] != w;
  }
  LaunchParams P;
  int rc = make_launch_params(params, &P);
  if (rc != SF_OK)
    return rc;
  const bool streamed16 = stream16_path(d_images, n, widths, P);
  const bool streamed = stream_path(sizeof(T), P) || streamed16;
  const WorkspaceLayout L = layout(h, w, capacity, streamed ? n : 1);
  if (ws_bytes < L.total)
    return SF_EBADARG;
  if (mixed && streamed && P.half != 3) {
    // The strip path of kernel sizes 2 and 4 takes one shape a launch: each
    // frame alone, into its slots (its workspace fits in the batch's).
    for (size_t j = 0; j < n; j++) {
      const T *one[1] = {d_images[j]};
      rc = threshold_frames_mixed<T>(one, 1, heights + j, widths + j, params,
                                     d_out + j * capacity, capacity, d_bits + j * L.words,
                                     d_counts + j,
                                     d_word_prefix ? d_word_prefix + j * L.words : nullptr, d_ws,
                                     ws_bytes, run_rows, stream);
      if (rc != SF_OK)
        return rc;
    }
    return SF_OK;
  }
  unsigned char *ws = static_cast<unsigned char *>(d_ws);
  if (streamed) {
    FramePtrs F;
    for (size_t j = 0; j < n; j++) {
      F.image[j] = reinterpret_cast<const uint32_t *>(d_images[j]);
      F.h[j] = (int)heights[j];
      F.w[j] = (int)widths[j];
    }
    StreamBuffers b;
    b.bits = d_bits;
    b.words = L.words;
    b.scr1 = reinterpret_cast<uint32_t *>(ws + L.scr1);
    b.amb = reinterpret_cast<uint32_t *>(ws + L.amb);
    b.prefix = d_word_prefix;
    b.cand = reinterpret_cast<uint32_t *>(ws + L.cand);
    b.res = reinterpret_cast<uint2 *>(ws + L.res);
    b.cand_cap = (uint32_t)L.cand_cap;
    b.counters = reinterpret_cast<uint32_t *>(ws + L.counters);
    b.wide = reinterpret_cast<uint4 *>(ws + L.wide);
    b.block_sums = reinterpret_cast<uint32_t *>(ws + L.block_sums);
    b.capacity = (uint32_t)capacity;
    b.out = d_out;
    b.out_stride = capacity;
    b.count_out = d_counts;
    const StreamMarks *marks = g_profiling && !t_capturing ? t_marks.arm() : nullptr;
    t_marks.staged = true;
    cudaError_t e =
        streamed16 ? launch_stream16(F, (int)n, (int)h, (int)w, P, b, run_rows, stream, marks)
                   : launch_stream(F, (int)n, (int)h, (int)w, P, b, run_rows, stream, marks);
    if (e != cudaSuccess)
      return fail(e, "launching the threshold");
    return SF_OK;
  }
  const StreamMarks *marks = g_profiling && !t_capturing ? t_marks.arm() : nullptr;
  t_marks.staged = false;
  if (marks)
    cudaEventRecord(marks->start, stream);
  // The tile path, one frame after another on the stream.
  for (size_t j = 0; j < n; j++) {
    FrameBuffers fb;
    fb.bits = d_bits + j * L.words;
    fb.staging = reinterpret_cast<sf_signal_pixel *>(ws + L.staging);
    fb.out = d_out + j * capacity;
    fb.word_prefix = d_word_prefix ? d_word_prefix + j * L.words : nullptr;
    fb.tile_base = reinterpret_cast<uint32_t *>(ws + L.tile_base);
    fb.row_total = reinterpret_cast<uint32_t *>(ws + L.row_total);
    fb.total = d_counts + j;
    fb.capacity = (uint32_t)capacity;
    cudaError_t e =
        launch_threshold<T>(d_images[j], (int)heights[j], (int)widths[j], P, fb, stream);
    if (e != cudaSuccess)
      return fail(e, "launching the threshold");
  }
  if (marks)
    cudaEventRecord(marks->order, stream);
  return SF_OK;
}

template <typename T>
static int threshold_device(const T *d_image, size_t h, size_t w,
                            const sf_threshold_params *params,
                            sf_signal_pixel *d_out, size_t capacity,
                            uint32_t *d_bits, uint32_t *d_count,
                            uint32_t *d_word_prefix, void *d_ws, size_t ws_bytes,
                            cudaStream_t stream) {
  if (!d_image)
    return SF_EBADARG;
  const T *images[1] = {d_image};
  return threshold_frames<T>(images, 1, h, w, params, d_out, capacity, d_bits, d_count,
                             d_word_prefix, d_ws, ws_bytes, 0, stream);
}

// ---------------------------------------------------------------------------
// The per-thread host-frame path (gpu::find<T>).
// ---------------------------------------------------------------------------

class Workspace {
public:
  ~Workspace() {
    if (stream_) {
      cudaStreamSynchronize(stream_);
      cudaStreamDestroy(stream_);
    }
    for (cudaEvent_t &ev : marks_)
      if (ev)
        cudaEventDestroy(ev);
    cudaFree(image_);
    cudaFree(bits_);
    cudaFree(out_);
    cudaFree(ws_);
    cudaFree(count_);
    if (host_count_)
      cudaFreeHost(host_count_);
    cudaFree(chunk_);
    cudaFree(narrow_);
    cudaFree(table_);
    cudaFree(scratch_);
    if (table_host_)
      cudaFreeHost(table_host_);
  }

  int open() {
    cudaError_t e;
    if (stream_)
      return SF_OK;
    if ((e = cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking)) != cudaSuccess)
      return fail(e, "cudaStreamCreate");
    // The small results read back: the count (word 0), the decoder's error
    // record (1-3), the narrowing's largest value (4), the decoder's block
    // counter (5, device only), a frame scan (words 6-13, four 64-bit
    // counts); the same layout on both sides.
    if ((e = cudaMalloc(&count_, kWords * sizeof(uint32_t))) != cudaSuccess)
      return fail(e, "cudaMalloc for the count");
    if ((e = cudaMallocHost(&host_count_, kWords * sizeof(uint32_t))) != cudaSuccess)
      return fail(e, "cudaMallocHost for the count");
    return SF_OK;
  }

  static constexpr int kWords = 16, kWorst = 4, kNext = 5, kScan = 6;
  unsigned long long *scan_words() {
    return reinterpret_cast<unsigned long long *>(count_ + kScan);
  }
  const unsigned long long *host_scan_words() const {
    return reinterpret_cast<const unsigned long long *>(host_count_ + kScan);
  }

  int reserve_narrow(size_t bytes) {
    return grow(&narrow_, &narrow_cap_, bytes, "cudaMalloc for the narrowed frame");
  }

  int reserve_image(size_t bytes) {
    int rc = open();
    return rc != SF_OK ? rc : grow(&image_, &image_cap_, bytes, "cudaMalloc for the frame");
  }

  // The decoder's buffers: the chunk's payload, its block table (and the
  // pinned copy it is uploaded from) and, for bitshuffle blocks larger than
  // a warp's buffer, a frame-sized scratch buffer.
  int reserve_decode(const ChunkPlan &plan) {
    int rc = open();
    if (rc != SF_OK)
      return rc;
    const size_t table_bytes = plan.blocks.size() * sizeof(DecodeBlock);
    if ((rc = grow(&chunk_, &chunk_cap_, plan.payload, "cudaMalloc for the chunk")) != SF_OK ||
        (rc = grow(&table_, &table_cap_, table_bytes, "cudaMalloc for the block table")) !=
            SF_OK ||
        (plan.scratch &&
         (rc = grow(&scratch_, &scratch_cap_, plan.frame_bytes, "cudaMalloc for the scratch")) !=
             SF_OK))
      return rc;
    if (table_bytes > table_host_cap_) {
      cudaStreamSynchronize(stream_);
      if (table_host_)
        cudaFreeHost(table_host_);
      table_host_ = nullptr;
      table_host_cap_ = 0;
      cudaError_t e = cudaMallocHost(&table_host_, table_bytes);
      if (e != cudaSuccess)
        return fail(e, "cudaMallocHost for the block table");
      table_host_cap_ = table_bytes;
    }
    return SF_OK;
  }

  // The chunk `data` (host) decoded into d_frame on the stream; the error
  // record lands in host_count_[1 .. 3] once the stream is idle.
  int decode(const uint8_t *data, const ChunkPlan &plan, uint8_t *d_frame) {
    cudaError_t e;
    const size_t table_bytes = plan.blocks.size() * sizeof(DecodeBlock);
    std::memcpy(table_host_, plan.blocks.data(), table_bytes);
    if ((e = cudaMemcpyAsync(chunk_, data + 12, plan.payload, cudaMemcpyHostToDevice,
                             stream_)) != cudaSuccess)
      return fail(e, "copying a chunk to the device");
    if ((e = cudaMemcpyAsync(table_, table_host_, table_bytes, cudaMemcpyHostToDevice,
                             stream_)) != cudaSuccess)
      return fail(e, "copying the block table to the device");
    if ((e = cudaMemsetAsync(count_ + 1, 0, 3 * sizeof(uint32_t), stream_)) != cudaSuccess ||
        (e = cudaMemsetAsync(count_ + kNext, 0, sizeof(uint32_t), stream_)) != cudaSuccess)
      return fail(e, "cudaMemsetAsync");
    if ((e = launch_decode(chunk_, table_, plan.blocks.size(), plan.element, d_frame,
                           scratch_, count_ + 1, count_ + kNext, stream_)) != cudaSuccess)
      return fail(e, "launching the decoder");
    if ((e = cudaMemcpyAsync(host_count_ + 1, count_ + 1, 3 * sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, stream_)) != cudaSuccess)
      return fail(e, "reading the decoder's status back");
    return SF_OK;
  }

  // After the stream is idle: SF_OK, or SF_EDATA with the reference's text.
  int decoded(const ChunkPlan &plan) const {
    if (host_count_[1] == kDecOk)
      return SF_OK;
    t_last_error = decode_error_text(plan, host_count_ + 1);
    return SF_EDATA;
  }

  int reserve(size_t image_bytes, size_t h, size_t w, size_t capacity) {
    cudaError_t e;
    int rc = open();
    if (rc != SF_OK)
      return rc;
    const size_t bits_bytes = words_per_row((int)w) * h * sizeof(uint32_t);
    const size_t ws_bytes = sf_workspace_bytes(h, w, capacity);
    const size_t out_bytes = capacity * sizeof(sf_signal_pixel);
    if (image_bytes <= image_cap_ && bits_bytes <= bits_cap_ &&
        ws_bytes <= ws_cap_ && out_bytes <= out_cap_)
      return SF_OK;
    // Nothing may be in flight when the buffers go (dext_cuda.cu:508-511).
    cudaStreamSynchronize(stream_);
    if (image_bytes > image_cap_) {
      cudaFree(image_);
      image_ = nullptr;
      image_cap_ = 0;
      if ((e = cudaMalloc(&image_, image_bytes)) != cudaSuccess)
        return fail(e, "cudaMalloc for the frame");
      image_cap_ = image_bytes;
    }
    if (bits_bytes > bits_cap_) {
      cudaFree(bits_);
      bits_ = nullptr;
      bits_cap_ = 0;
      if ((e = cudaMalloc(&bits_, bits_bytes)) != cudaSuccess)
        return fail(e, "cudaMalloc for the bitmask");
      bits_cap_ = bits_bytes;
    }
    if (ws_bytes > ws_cap_) {
      cudaFree(ws_);
      ws_ = nullptr;
      ws_cap_ = 0;
      if ((e = cudaMalloc(&ws_, ws_bytes)) != cudaSuccess)
        return fail(e, "cudaMalloc for the workspace");
      ws_cap_ = ws_bytes;
    }
    if (out_bytes > out_cap_) {
      cudaFree(out_);
      out_ = nullptr;
      out_cap_ = 0;
      if ((e = cudaMalloc(&out_, out_bytes)) != cudaSuccess)
        return fail(e, "cudaMalloc for the signal list");
      out_cap_ = out_bytes;
    }
    return SF_OK;
  }

  cudaEvent_t *marks() {
    if (!marks_[0])
      for (cudaEvent_t &ev : marks_)
        cudaEventCreate(&ev);
    return marks_;
  }

  template <typename P> int grow(P **p, size_t *cap, size_t bytes, const char *what) {
    if (bytes <= *cap)
      return SF_OK;
    // Nothing may be in flight when a buffer goes.
    cudaStreamSynchronize(stream_);
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), bytes);
    if (e != cudaSuccess)
      return fail(e, what);
    *cap = bytes;
    return SF_OK;
  }

  cudaStream_t stream_ = nullptr;
  void *image_ = nullptr;
  uint32_t *bits_ = nullptr;
  sf_signal_pixel *out_ = nullptr;
  void *ws_ = nullptr;
  uint32_t *count_ = nullptr;
  uint32_t *host_count_ = nullptr;
  uint8_t *chunk_ = nullptr, *scratch_ = nullptr;
  uint16_t *narrow_ = nullptr;
  size_t narrow_cap_ = 0;
  DecodeBlock *table_ = nullptr;
  void *table_host_ = nullptr;
  size_t image_cap_ = 0, bits_cap_ = 0, ws_cap_ = 0, out_cap_ = 0;
  size_t chunk_cap_ = 0, table_cap_ = 0, table_host_cap_ = 0, scratch_cap_ = 0;
  cudaEvent_t marks_[3] = {nullptr, nullptr, nullptr};
};

static Workspace &workspace() {
  static thread_local Workspace ws;
  return ws;
}

// Leaves the stream idle however find() is left (dext_cuda.cu:455-467).
struct StreamGuard {
  cudaStream_t s;
  ~StreamGuard() {
    if (s)
      cudaStreamSynchronize(s);
  }
};

// One host frame thresholded; with a chunk plan, `image` is the chunk and
// only it crosses the host link, decoded on the device. With `narrow` (T is
// uint16_t) the frame is 32-bit and is narrowed to 16 bits on the device
// before the threshold (--gpu-force, find_spots.cc:781-795); a frame with a
// valid count at or above 0xFFFD is refused with *offending set.
template <typename T>
static int find_host(const void *image, size_t h, size_t w,
                     const sf_threshold_params *params, sf_signal_pixel *out,
                     size_t capacity, size_t *found, const ChunkPlan *plan = nullptr,
                     bool narrow = false, uint32_t *offending = nullptr) {
  if (found)
    *found = 0;
  if (!image || !found || (!out && capacity) || !shape_ok(h, w))
    return SF_EBADARG;
  if (capacity > 0xffffffffu)
    capacity = 0xffffffffu;
  LaunchParams P;
  int rc = make_launch_params(params, &P);
  if (rc != SF_OK)
    return rc;
  const size_t bytes = h * w * (narrow ? sizeof(uint32_t) : sizeof(T));
  // The device list needs at least one record for the kernels' pointers.
  const size_t dcap = capacity ? capacity : 1;
  Workspace &ws = workspace();
  if ((rc = ws.reserve(bytes, h, w, dcap)) != SF_OK)
    return rc;
  const bool decode = plan && plan->algorithm != kChunkNone;
  if (decode && (rc = ws.reserve_decode(*plan)) != SF_OK)
    return rc;
  if (narrow && (rc = ws.reserve_narrow(h * w * sizeof(uint16_t))) != SF_OK)
    return rc;
  const cudaStream_t stream = ws.stream_;
  StreamGuard idle{stream};
  const bool timing = g_profiling;
  cudaEvent_t *marks = timing ? ws.marks() : nullptr;
  cudaError_t e;
  if (timing)
    cudaEventRecord(marks[0], stream);
  if (decode) {
    if ((rc = ws.decode(static_cast<const uint8_t *>(image), *plan,
                        static_cast<uint8_t *>(ws.image_))) != SF_OK)
      return rc;
  } else if ((e = cudaMemcpyAsync(ws.image_, image, bytes, cudaMemcpyHostToDevice, stream)) !=
             cudaSuccess) {
    return fail(e, "copying a frame to the device");
  }
  const T *frame = static_cast<const T *>(ws.image_);
  if (narrow) {
    if ((e = launch_narrow(static_cast<const uint32_t *>(ws.image_), h * w, ws.narrow_,
                           ws.count_ + Workspace::kWorst, stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(ws.host_count_ + Workspace::kWorst, ws.count_ + Workspace::kWorst,
                             sizeof(uint32_t), cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
      return fail(e, "narrowing the frame to 16 bits");
    frame = reinterpret_cast<const T *>(ws.narrow_);
  }
  if (timing)
    cudaEventRecord(marks[1], stream);
  rc = threshold_device<T>(frame, h, w, params, ws.out_, dcap, ws.bits_, ws.count_, nullptr,
                           ws.ws_, ws.ws_cap_, stream);
  if (rc != SF_OK)
    return rc;
  if (timing)
    cudaEventRecord(marks[2], stream);
  if ((e = cudaMemcpyAsync(ws.host_count_, ws.count_, sizeof(uint32_t),
                           cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
    return fail(e, "reading the signal count back");
  if ((e = cudaStreamSynchronize(stream)) != cudaSuccess)
    return fail(e, "cudaStreamSynchronize");
  if (decode && (rc = ws.decoded(*plan)) != SF_OK)
    return rc;
  if (narrow) {
    const uint32_t worst = ws.host_count_[Workspace::kWorst];
    if (offending)
      *offending = worst;
    if (worst >= 0xFFFDu) {  // narrow_to_16's test (find_spots.cc:181)
      t_last_error = "a count of " + std::to_string(worst) + ", too large for 16 bits";
      return SF_EDATA;
    }
  }
  const size_t n = *ws.host_count_;
  if (n == kCountFault) {
    t_last_error = "a bounded device wait ran out of time (a frame tile's load)";
    return SF_ECUDA;
  }
  *found = n;
  sf_stage_times times = {0, 0, 0, 0, 0, 0, 0};
  if (timing) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, marks[0], marks[1]);
    times.upload = ms;
    t_marks.collect(&times);
  }
  if (n > capacity) {
    if (timing)
      t_stage_times = times;
    return SF_EOVERFLOW;
  }
  if (n) {
    const auto t0 = std::chrono::steady_clock::now();
    if ((e = cudaMemcpyAsync(out, ws.out_, n * sizeof(sf_signal_pixel),
                             cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
      return fail(e, "copying the signal pixels back");
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess)
      return fail(e, "cudaStreamSynchronize");
    times.copy = std::chrono::duration<double, std::milli>(
                     std::chrono::steady_clock::now() - t0)
                     .count();
  }
  if (timing)
    t_stage_times = times;
  return SF_OK;
}

} // namespace sf

using namespace sf;

extern "C" {

void sf_default_params(sf_threshold_params *p) {
  if (!p)
    return;
  p->algorithm = SF_DISPERSION_EXTENDED;
  p->kernel_x = 3;
  p->kernel_y = 3;
  p->gain = 1.0;
  p->sigma_b = 6.0;
  p->sigma_s = 3.0;
  p->min_local = 2;
  p->global_threshold = 0.0;
}

const char *sf_backend(void) { return "CUDA (GB300, sm_103a)"; }

static std::once_flag g_probe_once;
static int g_available = 0;
static std::string g_reason;

static void probe() {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess) {
    g_reason = std::string("no CUDA device: ") + cudaGetErrorString(e);
    return;
  }
  if (count == 0) {
    g_reason = "no CUDA device";
    return;
  }
  int dev = 0, major = 0, minor = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10 || minor != 3) {
    char buf[128];
    std::snprintf(buf, sizeof(buf),
                  "device %d is compute capability %d.%d; this build is sm_103a only",
                  dev, major, minor);
    g_reason = buf;
    return;
  }
  g_available = 1;
}

int sf_available(void) {
  std::call_once(g_probe_once, probe);
  return g_available;
}

const char *sf_unavailable_reason(void) {
  std::call_once(g_probe_once, probe);
  return g_available ? "" : g_reason.c_str();
}

size_t sf_memory_free(void) {
  size_t free_b = 0, total = 0;
  if (cudaMemGetInfo(&free_b, &total) != cudaSuccess)
    return 0;
  return free_b;
}

void *sf_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess)
    return nullptr;
  return p;
}

void sf_host_free(void *pointer) {
  if (pointer)
    cudaFreeHost(pointer);
}

const char *sf_last_error(void) { return t_last_error.c_str(); }

int sf_find_u32(const uint32_t *image, size_t height, size_t width,
                sf_signal_pixel *out, size_t capacity, size_t *found) {
  return find_host<uint32_t>(image, height, width, nullptr, out, capacity, found);
}
int sf_find_u16(const uint16_t *image, size_t height, size_t width,
                sf_signal_pixel *out, size_t capacity, size_t *found) {
  return find_host<uint16_t>(image, height, width, nullptr, out, capacity, found);
}
int sf_find_u32_params(const uint32_t *image, size_t height, size_t width,
                       const sf_threshold_params *params, sf_signal_pixel *out,
                       size_t capacity, size_t *found) {
  return find_host<uint32_t>(image, height, width, params, out, capacity, found);
}
int sf_find_u16_params(const uint16_t *image, size_t height, size_t width,
                       const sf_threshold_params *params, sf_signal_pixel *out,
                       size_t capacity, size_t *found) {
  return find_host<uint16_t>(image, height, width, params, out, capacity, found);
}

size_t sf_frame_bytes(size_t height, size_t width, unsigned bit_depth) {
  return height * width * bit_depth / 8;
}

// decompress::image into host (to_device false) or device memory.
static int decompress_to(const uint8_t *data, size_t nbytes, const char *algorithm,
                         unsigned bit_depth, size_t height, size_t width, void *out,
                         size_t out_bytes, bool to_device) {
  if ((!data && nbytes) || !out || !shape_ok(height, width) || bit_depth > 64)
    return SF_EBADARG;
  if (to_device && reinterpret_cast<uintptr_t>(out) % 16 != 0) {
    t_last_error = "the device frame must be 16-byte aligned";
    return SF_EBADARG;
  }
  ChunkPlan plan;
  int rc = plan_chunk(data, nbytes, algorithm, bit_depth, height, width, out_bytes, &plan);
  if (rc != SF_OK)
    return rc;
  if (plan.algorithm == kChunkNone && !to_device) {
    std::memcpy(out, data, nbytes);  // decompress.cc:93
    return SF_OK;
  }
  Workspace &ws = workspace();
  if ((rc = to_device ? ws.open() : ws.reserve_image(plan.frame_bytes)) != SF_OK)
    return rc;
  uint8_t *frame = static_cast<uint8_t *>(to_device ? out : ws.image_);
  const cudaStream_t stream = ws.stream_;
  StreamGuard idle{stream};
  cudaError_t e;
  if (plan.algorithm == kChunkNone) {
    if ((e = cudaMemcpyAsync(frame, data, nbytes, cudaMemcpyHostToDevice, stream)) !=
        cudaSuccess)
      return fail(e, "copying a frame to the device");
  } else {
    if ((rc = ws.reserve_decode(plan)) != SF_OK || (rc = ws.decode(data, plan, frame)) != SF_OK)
      return rc;
    if (!to_device && (e = cudaMemcpyAsync(out, frame, plan.frame_bytes, cudaMemcpyDeviceToHost,
                                           stream)) != cudaSuccess)
      return fail(e, "copying the frame back");
  }
  if ((e = cudaStreamSynchronize(stream)) != cudaSuccess)
    return fail(e, "cudaStreamSynchronize");
  return plan.algorithm == kChunkNone ? SF_OK : ws.decoded(plan);
}

int sf_decompress_image(const uint8_t *data, size_t nbytes, const char *algorithm,
                        unsigned bit_depth, size_t height, size_t width, uint8_t *out,
                        size_t out_bytes) {
  return decompress_to(data, nbytes, algorithm, bit_depth, height, width, out, out_bytes,
                       false);
}

int sf_decompress_device(const uint8_t *data, size_t nbytes, const char *algorithm,
                         unsigned bit_depth, size_t height, size_t width, void *d_out,
                         size_t out_bytes) {
  return decompress_to(data, nbytes, algorithm, bit_depth, height, width, d_out, out_bytes,
                       true);
}

int sf_find_compressed(const uint8_t *data, size_t nbytes, const char *algorithm,
                       unsigned bit_depth, size_t height, size_t width,
                       const sf_threshold_params *params, sf_signal_pixel *out,
                       size_t capacity, size_t *found) {
  if (found)
    *found = 0;
  if (!data || !found || (!out && capacity) || !shape_ok(height, width))
    return SF_EBADARG;
  if (bit_depth != 16 && bit_depth != 32) {
    t_last_error = "frames of 16- or 32-bit pixels are thresholded";
    return SF_EUNSUPPORTED;
  }
  ChunkPlan plan;
  const size_t frame = height * width * bit_depth / 8;
  int rc = plan_chunk(data, nbytes, algorithm, bit_depth, height, width, frame, &plan);
  if (rc != SF_OK)
    return rc;
  return bit_depth == 16
             ? find_host<uint16_t>(data, height, width, params, out, capacity, found, &plan)
             : find_host<uint32_t>(data, height, width, params, out, capacity, found, &plan);
}

int sf_find_narrowed(const uint8_t *data, size_t nbytes, const char *algorithm, size_t height,
                     size_t width, const sf_threshold_params *params, sf_signal_pixel *out,
                     size_t capacity, size_t *found, uint32_t *offending) {
  if (found)
    *found = 0;
  if (offending)
    *offending = 0;
  if (!data || !found || (!out && capacity) || !shape_ok(height, width))
    return SF_EBADARG;
  ChunkPlan plan;
  int rc = plan_chunk(data, nbytes, algorithm, 32, height, width, height * width * 4, &plan);
  if (rc != SF_OK)
    return rc;
  return find_host<uint16_t>(data, height, width, params, out, capacity, found, &plan, true,
                             offending);
}

int sf_scan_device(const void *d_image, size_t n_pixels, unsigned bit_depth,
                   sf_frame_scan *out) {
  if ((!d_image && n_pixels) || !out || (bit_depth != 16 && bit_depth != 32) ||
      n_pixels > 0x7fffffffu)
    return SF_EBADARG;
  if (n_pixels == 0) {
    *out = {0, 0, 0, 0};
    return SF_OK;
  }
  Workspace &ws = workspace();
  int rc = ws.open();
  if (rc != SF_OK)
    return rc;
  const cudaStream_t stream = ws.stream_;
  StreamGuard idle{stream};
  cudaError_t e;
  if ((e = launch_scan(d_image, n_pixels, bit_depth, ws.scan_words(), stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(ws.host_count_ + Workspace::kScan, ws.scan_words(),
                           4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(stream)) != cudaSuccess)
    return fail(e, "scanning the frame");
  const unsigned long long *r = ws.host_scan_words();
  *out = {r[0], r[1], r[2], r[3]};
  return SF_OK;
}

int sf_scan_compressed(const uint8_t *data, size_t nbytes, const char *algorithm,
                       unsigned bit_depth, size_t height, size_t width, sf_frame_scan *out) {
  if (!data || !out || !shape_ok(height, width))
    return SF_EBADARG;
  if (bit_depth != 16 && bit_depth != 32) {
    t_last_error = std::to_string(bit_depth) + "-bit pixels";  // mxi_max.cc:165-166
    return SF_EUNSUPPORTED;
  }
  ChunkPlan plan;
  const size_t bytes = height * width * bit_depth / 8;
  int rc = plan_chunk(data, nbytes, algorithm, bit_depth, height, width, bytes, &plan);
  if (rc != SF_OK)
    return rc;
  Workspace &ws = workspace();
  if ((rc = ws.reserve_image(bytes)) != SF_OK)
    return rc;
  const cudaStream_t stream = ws.stream_;
  StreamGuard idle{stream};
  cudaError_t e;
  const bool decode = plan.algorithm != kChunkNone;
  if (decode) {
    if ((rc = ws.reserve_decode(plan)) != SF_OK ||
        (rc = ws.decode(data, plan, static_cast<uint8_t *>(ws.image_))) != SF_OK)
      return rc;
  } else if ((e = cudaMemcpyAsync(ws.image_, data, bytes, cudaMemcpyHostToDevice, stream)) !=
             cudaSuccess) {
    return fail(e, "copying a frame to the device");
  }
  if ((e = launch_scan(ws.image_, height * width, bit_depth, ws.scan_words(), stream)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(ws.host_count_ + Workspace::kScan, ws.scan_words(),
                           4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(stream)) != cudaSuccess)
    return fail(e, "scanning the frame");
  if (decode && (rc = ws.decoded(plan)) != SF_OK)
    return rc;
  const unsigned long long *r = ws.host_scan_words();
  *out = {r[0], r[1], r[2], r[3]};
  return SF_OK;
}

void sf_profile_stages(int on) { g_profiling = on != 0; }
int sf_profiling(void) { return g_profiling ? 1 : 0; }
void sf_last_stage_times(sf_stage_times *out) {
  t_marks.collect(&t_stage_times);
  if (out)
    *out = t_stage_times;
}

size_t sf_workspace_bytes(size_t height, size_t width, size_t capacity) {
  if (!shape_ok(height, width))
    return 0;
  return layout(height, width, capacity).total;
}

int sf_threshold_u32_device(const uint32_t *d_image, size_t height, size_t width,
                            const sf_threshold_params *params,
                            sf_signal_pixel *d_out, size_t capacity,
                            uint32_t *d_bits, uint32_t *d_count,
                            uint32_t *d_word_prefix, void *d_workspace,
                            size_t workspace_bytes, void *stream) {
  return threshold_device<uint32_t>(d_image, height, width, params, d_out, capacity,
                                    d_bits, d_count, d_word_prefix, d_workspace,
                                    workspace_bytes, static_cast<cudaStream_t>(stream));
}

int sf_threshold_u16_device(const uint16_t *d_image, size_t height, size_t width,
                            const sf_threshold_params *params,
                            sf_signal_pixel *d_out, size_t capacity,
                            uint32_t *d_bits, uint32_t *d_count,
                            uint32_t *d_word_prefix, void *d_workspace,
                            size_t workspace_bytes, void *stream) {
  return threshold_device<uint16_t>(d_image, height, width, params, d_out, capacity,
                                    d_bits, d_count, d_word_prefix, d_workspace,
                                    workspace_bytes, static_cast<cudaStream_t>(stream));
}

size_t sf_batch_workspace_bytes(size_t n_frames, size_t height, size_t width,
                                size_t capacity) {
  if (!shape_ok(height, width) || n_frames == 0 || n_frames > (size_t)kMaxBatch)
    return 0;
  return layout(height, width, capacity, n_frames).total;
}

int sf_threshold_u32_batch_device(const uint32_t *const *d_images, size_t n_frames,
                                  size_t height, size_t width,
                                  const sf_threshold_params *params, sf_signal_pixel *d_out,
                                  size_t capacity, uint32_t *d_bits, uint32_t *d_counts,
                                  uint32_t *d_word_prefix, void *d_workspace,
                                  size_t workspace_bytes, void *stream) {
  return threshold_frames<uint32_t>(d_images, n_frames, height, width, params, d_out, capacity,
                                    d_bits, d_counts, d_word_prefix, d_workspace,
                                    workspace_bytes, 0, static_cast<cudaStream_t>(stream));
}

int sf_threshold_u16_batch_device(const uint16_t *const *d_images, size_t n_frames,
                                  size_t height, size_t width,
                                  const sf_threshold_params *params, sf_signal_pixel *d_out,
                                  size_t capacity, uint32_t *d_bits, uint32_t *d_counts,
                                  uint32_t *d_word_prefix, void *d_workspace,
                                  size_t workspace_bytes, void *stream) {
  return threshold_frames<uint16_t>(d_images, n_frames, height, width, params, d_out, capacity,
                                    d_bits, d_counts, d_word_prefix, d_workspace,
                                    workspace_bytes, 0, static_cast<cudaStream_t>(stream));
}

size_t sf_mixed_batch_workspace_bytes(size_t n_frames, const size_t *heights,
                                      const size_t *widths, size_t capacity) {
  size_t h = 0, w = 0;
  if (!heights || !widths || n_frames == 0 || n_frames > (size_t)kMaxBatch ||
      !envelope(n_frames, heights, widths, &h, &w))
    return 0;
  return layout(h, w, capacity, n_frames).total;
}

size_t sf_mixed_batch_mask_words(size_t n_frames, const size_t *heights, const size_t *widths) {
  size_t h = 0, w = 0;
  if (!heights || !widths || n_frames == 0 || n_frames > (size_t)kMaxBatch ||
      !envelope(n_frames, heights, widths, &h, &w))
    return 0;
  return (w + 31) / 32 * h;
}

int sf_threshold_u32_mixed_batch_device(const uint32_t *const *d_images, const size_t *heights,
                                        const size_t *widths, size_t n_frames,
                                        const sf_threshold_params *params,
                                        sf_signal_pixel *d_out, size_t capacity,
                                        uint32_t *d_bits, uint32_t *d_counts,
                                        uint32_t *d_word_prefix, void *d_workspace,
                                        size_t workspace_bytes, void *stream) {
  return threshold_frames_mixed<uint32_t>(d_images, n_frames, heights, widths, params, d_out,
                                          capacity, d_bits, d_counts, d_word_prefix,
                                          d_workspace, workspace_bytes, 0,
                                          static_cast<cudaStream_t>(stream));
}

} // extern "C"

// ---------------------------------------------------------------------------
// The device threshold for callers that cannot allocate device memory.
//
// Some callers may not call cudaMalloc at all: a plugin running inside a host
// application whose own allocator owns every byte of device memory, or a
// detector-stream loop that must not stall acquisition on the device-wide
// synchronisation an allocation can cause. For them the threshold's scratch
// (the unordered signal list, the per-tile bases and the per-tile-row counts)
// lives in a fixed array in this library's device image instead of a
// caller-supplied workspace. The array is part of the module that holds this
// file's code: the driver reserves it on a device when that module is first
// loaded there (under CUDA's lazy module loading, at the first use of the
// module on that device, at the latest at this entry point's first call) and
// keeps it until the process exits.
// ---------------------------------------------------------------------------

namespace sf {

// 32 MiB. What one call needs is the workspace layout of (height, width,
// capacity): the tile path's staging list (16 bytes a record), the candidate
// list and stage-2 results (12 bytes a slot, min(h w, 2 capacity + 65536)
// slots), the eroded mask, word prefixes and tile bookkeeping. A call is
// refused unless that layout fits. It does at the full 524,288 records for an
// EIGER2 16M frame (4362 x 4148: 27.2 MB) and for every frame of up to 2^25
// pixels whose sides are both at least 256 (at most 31.7 MB).
constexpr size_t kNoAllocCapacity = 524288;
constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The device address of g_noalloc_scratch, looked up once per device. In host
// code the array's name only stands in for the symbol; its address on the
// device comes from cudaGetSymbolAddress, with that device current.
constexpr int kNoAllocMaxDevices = 64;
static void *g_noalloc_ptr[kNoAllocMaxDevices] = {};
static std::mutex g_noalloc_mutex;

static int noalloc_scratch(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    t_last_error = "device index beyond the scratch table";
    return SF_EBADARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(e, "cudaGetSymbolAddress for the fixed scratch");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return SF_OK;
}

} // namespace sf

extern "C" int sf_threshold_u32_device_noalloc(
    const uint32_t *d_image, size_t height, size_t width,
    const sf_threshold_params *params, sf_signal_pixel *d_out, size_t capacity,
    uint32_t *d_bits, uint32_t *d_count, uint32_t *d_word_prefix, void *stream) {
  using namespace sf;
  if (!shape_ok(height, width))
    return SF_EBADARG;
  if (capacity > kNoAllocCapacity) {
    t_last_error = "capacity above the fixed scratch's 524288 records";
    return SF_EBADARG;
  }
  if (layout(height, width, capacity).total > kNoAllocScratchBytes) {
    t_last_error = "frame and capacity together need more than the fixed scratch's 32 MiB";
    return SF_EBADARG;
  }
  void *scratch = nullptr;
  const int rc = noalloc_scratch(&scratch);
  if (rc != SF_OK)
    return rc;
  // threshold_device clears the per-tile-row counts and the total on the
  // stream before the kernels run; the staging list and tile bases are
  // written before they are read, so nothing else needs to start at zero.
  return threshold_device<uint32_t>(d_image, height, width, params, d_out, capacity,
                                    d_bits, d_count, d_word_prefix, scratch,
                                    kNoAllocScratchBytes,
                                    static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------------------
// Batch plans: one frame shape, its outputs and workspace, a run length tuned
// on real frames, and the launch sequence captured as CUDA graphs, replayed
// whenever the same frame buffers come again (a detector loop cycles a fixed
// set of them).
// ---------------------------------------------------------------------------

namespace sf {

constexpr size_t kPlanMaxGraphs = 16;

struct Plan {
  size_t h = 0, w = 0, max_frames = 0, capacity = 0, words = 0;
  sf_threshold_params params{};
  int run_rows = 0;  // 0: the default geometry
  // Frames a launch sequence takes (0: all of a call's frames in one); a
  // call of more runs as consecutive sequences on its stream.
  size_t per_launch = 0;
  void *ws = nullptr;
  size_t ws_bytes = 0;
  sf_signal_pixel *lists = nullptr;
  uint32_t *masks = nullptr, *counts = nullptr;
  cudaStream_t capture = nullptr;
  struct Graph {
    std::vector<const uint32_t *> frames;
    cudaGraphExec_t exec = nullptr;
  };
  std::vector<Graph> graphs;  // most recently made last
  bool warm = false;

  ~Plan() {
    drop_graphs();
    if (capture)
      cudaStreamDestroy(capture);
    cudaFree(ws);
    cudaFree(lists);
    cudaFree(masks);
    cudaFree(counts);
  }
  void drop_graphs() {
    for (Graph &g : graphs)
      cudaGraphExecDestroy(g.exec);
    graphs.clear();
  }
  int launch(const uint32_t *const *images, size_t n, cudaStream_t s) {
    const size_t step = per_launch ? per_launch : n;
    for (size_t j = 0; j < n; j += step) {
      const size_t m = std::min(step, n - j);
      const int rc = threshold_frames<uint32_t>(images + j, m, h, w, &params, lists + j * capacity,
                                                capacity, masks + j * words, counts + j, nullptr,
                                                ws, ws_bytes, run_rows, s);
      if (rc != SF_OK)
        return rc;
    }
    return SF_OK;
  }
};

static int plan_run(Plan &pl, const uint32_t *const *images, size_t n, cudaStream_t s) {
  if (!images || n == 0 || n > pl.max_frames)
    return SF_EBADARG;
  if (!pl.warm) {
    // The first launch runs directly: one-time set-up (kernel attributes,
    // occupancy queries) stays outside any capture.
    const int rc = pl.launch(images, n, s);
    pl.warm = rc == SF_OK;
    return rc;
  }
  for (size_t i = 0; i < pl.graphs.size(); i++) {
    Plan::Graph &g = pl.graphs[i];
    if (g.frames.size() == n && std::equal(g.frames.begin(), g.frames.end(), images)) {
      const cudaError_t e = cudaGraphLaunch(g.exec, s);
      return e == cudaSuccess ? SF_OK : fail(e, "cudaGraphLaunch");
    }
  }
  cudaError_t e;
  if ((e = cudaStreamBeginCapture(pl.capture, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return fail(e, "cudaStreamBeginCapture");
  t_capturing = true;
  const int rc = pl.launch(images, n, pl.capture);
  t_capturing = false;
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(pl.capture, &graph);
  if (rc != SF_OK) {
    if (graph)
      cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess)
    return fail(e, "cudaStreamEndCapture");
  Plan::Graph g;
  g.frames.assign(images, images + n);
  e = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess)
    return fail(e, "cudaGraphInstantiate");
  if (pl.graphs.size() == kPlanMaxGraphs) {
    cudaGraphExecDestroy(pl.graphs.front().exec);
    pl.graphs.erase(pl.graphs.begin());
  }
  pl.graphs.push_back(std::move(g));
  e = cudaGraphLaunch(pl.graphs.back().exec, s);
  return e == cudaSuccess ? SF_OK : fail(e, "cudaGraphLaunch");
}

} // namespace sf

struct sf_plan {
  sf::Plan impl;
};

extern "C" {

sf_plan *sf_plan_create(size_t height, size_t width, size_t max_frames, size_t capacity,
                        const sf_threshold_params *params) {
  using namespace sf;
  if (!shape_ok(height, width) || max_frames == 0 || max_frames > (size_t)kMaxBatch ||
      capacity == 0 || capacity > 0xffffffffu) {
    t_last_error = "plan: bad shape, batch size or capacity";
    return nullptr;
  }
  LaunchParams P;
  if (make_launch_params(params, &P) != SF_OK) {
    t_last_error = "plan: threshold parameters refused";
    return nullptr;
  }
  sf_plan *pl = new sf_plan();
  Plan &p = pl->impl;
  p.h = height;
  p.w = width;
  p.max_frames = max_frames;
  p.capacity = capacity;
  p.words = (width + 31) / 32 * height;
  if (params)
    p.params = *params;
  else
    sf_default_params(&p.params);
  p.ws_bytes = sf_batch_workspace_bytes(max_frames, height, width, capacity);
  cudaError_t e;
  if ((e = cudaMalloc(&p.ws, p.ws_bytes)) != cudaSuccess ||
      (e = cudaMalloc(&p.lists, max_frames * capacity * sizeof(sf_signal_pixel))) !=
          cudaSuccess ||
      (e = cudaMalloc(&p.masks, max_frames * p.words * sizeof(uint32_t))) != cudaSuccess ||
      (e = cudaMalloc(&p.counts, max_frames * sizeof(uint32_t))) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&p.capture, cudaStreamNonBlocking)) != cudaSuccess) {
    fail(e, "plan: device buffers");
    delete pl;
    return nullptr;
  }
  return pl;
}

void sf_plan_destroy(sf_plan *plan) {
  if (!plan)
    return;
  cudaDeviceSynchronize();
  delete plan;
}

int sf_plan_run(sf_plan *plan, const uint32_t *const *d_images, size_t n_frames, void *stream) {
  if (!plan)
    return SF_EBADARG;
  return sf::plan_run(plan->impl, d_images, n_frames, static_cast<cudaStream_t>(stream));
}

int sf_plan_tune(sf_plan *plan, const uint32_t *const *d_images, size_t n_frames, void *stream) {
  using namespace sf;
  if (!plan || !d_images || n_frames == 0 || n_frames > plan->impl.max_frames)
    return SF_EBADARG;
  Plan &p = plan->impl;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  LaunchParams P;
  int rc = make_launch_params(&p.params, &P);
  if (rc != SF_OK)
    return rc;
  if (P.algorithm != SF_DISPERSION_EXTENDED || !P.int_ok)
    return SF_OK;  // the tile path has nothing to tune
  // Two knobs, timed together on the given frames (median of 3 runs each):
  // the frames a launch sequence takes (all of them, 32 or 16: fewer frames
  // a launch keep more of a batch's tiles in L2 between the passes, more
  // frames fill the GPU with fewer launches) and, for each, the strip run
  // length around its default geometry.
  std::vector<size_t> per = {n_frames};
  for (size_t q : {(size_t)32, (size_t)16})
    if (q < n_frames && n_frames % q == 0)
      per.push_back(q);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best_ms = 1e30f;
  int best = 0;
  size_t best_per = 0;
  for (size_t q : per) {
    const int base = stream_default_run_rows(P, (int)p.h, (int)p.w, (int)q);
    std::vector<int> cands = {base, base / 2, base / 3, base / 4, 2 * base, 64, 128, 256, 512};
    std::sort(cands.begin(), cands.end());
    cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
    p.per_launch = q == n_frames ? 0 : q;
    for (int rr : cands) {
      if (rr < kMinRunRows || rr > (int)p.h)
        continue;
      p.run_rows = rr;
      float ms[3];
      for (int it = 0; it < 4; it++) {
        cudaEventRecord(a, s);
        if ((rc = p.launch(d_images, n_frames, s)) != SF_OK)
          break;
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        if (it)
          cudaEventElapsedTime(&ms[it - 1], a, b);
      }
      if (rc != SF_OK)
        break;
      std::sort(ms, ms + 3);
      if (ms[1] < best_ms) {
        best_ms = ms[1];
        best = rr;
        best_per = p.per_launch;
      }
    }
    if (rc != SF_OK)
      break;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  p.run_rows = best;
  p.per_launch = best_per;
  p.drop_graphs();
  p.warm = true;
  return rc;
}

int sf_plan_run_rows(const sf_plan *plan) { return plan ? plan->impl.run_rows : 0; }
size_t sf_plan_frames_per_launch(const sf_plan *plan) {
  return plan ? plan->impl.per_launch : 0;
}

int sf_plan_configure(sf_plan *plan, int run_rows, size_t frames_per_launch) {
  using namespace sf;
  if (!plan || run_rows < 0 || frames_per_launch > plan->impl.max_frames)
    return SF_EBADARG;
  Plan &p = plan->impl;
  p.run_rows = run_rows;
  p.per_launch = frames_per_launch;
  p.drop_graphs();
  return SF_OK;
}
size_t sf_plan_graphs(const sf_plan *plan) { return plan ? plan->impl.graphs.size() : 0; }
sf_signal_pixel *sf_plan_lists(const sf_plan *plan) { return plan ? plan->impl.lists : nullptr; }
uint32_t *sf_plan_counts(const sf_plan *plan) { return plan ? plan->impl.counts : nullptr; }
uint32_t *sf_plan_masks(const sf_plan *plan) { return plan ? plan->impl.masks : nullptr; }

int sf_plan_result(sf_plan *plan, size_t j, sf_signal_pixel *out, size_t capacity,
                   size_t *found) {
  using namespace sf;
  if (found)
    *found = 0;
  if (!plan || !found || j >= plan->impl.max_frames || (!out && capacity))
    return SF_EBADARG;
  Plan &p = plan->impl;
  cudaError_t e;
  if ((e = cudaDeviceSynchronize()) != cudaSuccess)
    return fail(e, "cudaDeviceSynchronize");
  uint32_t n = 0;
  if ((e = cudaMemcpy(&n, p.counts + j, sizeof(n), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return fail(e, "reading a plan's count");
  if (n == kCountFault) {
    t_last_error = "a bounded device wait ran out of time (a frame tile's load)";
    return SF_ECUDA;
  }
  *found = n;
  if (n > p.capacity || n > capacity)
    return SF_EOVERFLOW;
  if (n && (e = cudaMemcpy(out, p.lists + j * p.capacity, n * sizeof(sf_signal_pixel),
                           cudaMemcpyDeviceToHost)) != cudaSuccess)
    return fail(e, "reading a plan's list");
  return SF_OK;
}

} // extern "C"
