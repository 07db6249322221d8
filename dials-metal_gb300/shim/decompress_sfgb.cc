// decompress::frame_bytes and decompress::image (src/spots/decompress.hh:17-31,
// decompress.cc:72-134) over libsfgb: the chunk is decoded on the device and
// the frame copied back to `out`. Links in place of decompress.cc, with no
// bitshuffle or lz4 library. The reference's exception texts come back
// through sf_last_error().
//
// A worker that thresholds right after decoding gains more from
// sf_find_compressed, which sends only the chunk over the host link and never
// brings the frame back.

#include <cstddef>
#include <cstdint>
#include <span>
#include <stdexcept>
#include <string>
#include <string_view>

#include "decompress.hh"
#include "sf_api.h"

namespace decompress {

std::size_t frame_bytes(std::size_t height, std::size_t width, unsigned bit_depth) {
  return sf_frame_bytes(height, width, bit_depth);
}

void image(std::span<const std::uint8_t> data, std::string_view algorithm, unsigned bit_depth,
           std::size_t height, std::size_t width, std::span<std::uint8_t> out) {
  const std::string name(algorithm);
  const int rc = sf_decompress_image(data.data(), data.size(), name.c_str(), bit_depth, height,
                                     width, out.data(), out.size());
  if (rc != SF_OK)
    throw std::runtime_error(sf_last_error());
}

} // namespace decompress
