// Internal interface of the threshold kernels (sf_threshold.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sf_common.cuh"

namespace sf {

// Output tile of one threshold block: 32 columns (one bitmask word) by 32 rows.
constexpr int kTileW = 32;
constexpr int kTileH = 32;

// Device buffers of one threshold launch. All are device pointers.
struct FrameBuffers {
  uint32_t *bits;            // ceil(W/32) words per row, H rows
  sf_signal_pixel *staging;  // `capacity` records, tile order
  sf_signal_pixel *out;      // `capacity` records, ascending index
  uint32_t *word_prefix;     // optional: exclusive popcount prefix per word
  uint32_t *total;           // one word: signal pixels found
  uint32_t *row_total;       // tiles_y entries: signal per tile row
  uint32_t *tile_base;       // tiles_x * tiles_y entries
  uint32_t capacity;
};

inline int tiles_x(int w) { return (w + kTileW - 1) / kTileW; }
inline int tiles_y(int h) { return (h + kTileH - 1) / kTileH; }
inline size_t words_per_row(int w) { return (size_t)((w + 31) / 32); }

size_t order_smem_bytes(int width);

template <typename T>
cudaError_t launch_threshold(const T *image, int h, int w, const LaunchParams &P,
                             const FrameBuffers &fb, cudaStream_t stream);

} // namespace sf
