// Whole-frame passes around the threshold (sf_frames.cu): mxi_max's scan
// and the --gpu-force narrowing to 16 bits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sf {

// mxi_max's scan<T> (apps/mxi_max.cc:47-67) of n pixels of bit_depth 16 or
// 32 into d_out[4] = {largest non-marker value, bad pixels, tile joins,
// valid pixels at 0xFFFD or above}; d_out is zeroed first on the stream.
cudaError_t launch_scan(const void *d_image, size_t n, unsigned bit_depth,
                        unsigned long long *d_out, cudaStream_t stream);

// narrow_to_16 (find_spots.cc:169-182): d_out[i] = the low 16 bits of
// d_in[i]; *d_worst = the largest value below the 32-bit markers.
cudaError_t launch_narrow(const uint32_t *d_in, size_t n, uint16_t *d_out, uint32_t *d_worst,
                          cudaStream_t stream);

}  // namespace sf
