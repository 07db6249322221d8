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

// The served form's hold on a labeller's result storage: ok(ctx, bytes) is
// asked before each new device chunk of the spot and pixel stores; when it
// says no, the add that needed the room returns SF_EBUSY and the store does
// not grow.
struct LabelGrowth {
  bool (*ok)(void *ctx, size_t bytes) = nullptr;
  void *ctx = nullptr;
};
void label_set_growth(sf_labeller *labeller, LabelGrowth growth);
// Device bytes the labeller's spot and pixel stores hold now.
size_t label_result_bytes(const sf_labeller *labeller);
// Waits for the end of each call sleeping on a blocking-sync event instead
// of spinning in a stream synchronisation.
int label_set_blocking_wait(sf_labeller *labeller);
// Captures every call shape of up to max_batch frames now (see
// Labeller::prepare in sf_label.cu). SF_OK or SF_ECUDA.
int label_prepare(sf_labeller *labeller, int max_batch);

} // namespace sf
