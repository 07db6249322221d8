// Internal constants of the device labeller (sf_label.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "sf_api.h"

namespace sf {

// Frames labelled together in one batch.
constexpr int kLabelMaxBatch = 64;

// For the reflection-table writer (sf_refl.cu): the frame width a labeller
// was opened with, and its kept pixels gathered into one device buffer of
// sf_label_n_pixels elements by device-to-device copies on the labeller's own
// stream, after its last add; *stream is that stream. 0 or SF_ECUDA.
size_t label_width(const sf_labeller *labeller);
int label_gather_pixels(const sf_labeller *labeller, sf_pixel *d_out, cudaStream_t *stream);

// Device bytes sf_label_open(height, ., options, capacity) allocates before
// any result is stored: pools, scratch, row tables and batch outputs.
size_t label_device_bytes(size_t height, size_t capacity, size_t min_spot_size);

} // namespace sf
