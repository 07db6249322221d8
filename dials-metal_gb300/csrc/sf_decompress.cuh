// Frame decompression on the device: decompress::image
// (src/spots/decompress.cc:77-134) for chunks stored bitshuffle+LZ4
// ("bslz4"), LZ4 ("lz4") or uncompressed (""), decoded where the threshold
// reads them.
//
// The host reads the 12-byte filter header and walks the chunk's block
// framing (a dependent chain of 4-byte lengths) into a table of blocks; the
// device decodes every block at once, one warp a block.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace sf {

enum DecodeMode : uint32_t {
  kDecLz4 = 0,         // an LZ4 block decoded straight into the frame
  kDecBitshuffle = 1,  // an LZ4 block of bit planes, then transposed into the frame
  kDecRaw = 2,         // bytes copied as they are (bitshuffle's size % 8 tail)
};

// One block of a chunk: where it starts in the payload (after the filter
// header), where its bytes go in the frame, and their counts.
struct DecodeBlock {
  unsigned long long in_off, out_off;
  uint32_t in_bytes, out_bytes, elems, mode;
};

enum ChunkAlgorithm { kChunkNone = 0, kChunkLz4 = 1, kChunkBitshuffle = 2 };

struct ChunkPlan {
  ChunkAlgorithm algorithm = kChunkNone;
  size_t frame_bytes = 0;   // decoded bytes: height x width x element
  unsigned element = 0;     // bytes a pixel
  size_t payload = 0;       // bytes after the filter header
  std::vector<DecodeBlock> blocks;
  bool scratch = false;     // some bitshuffle block is larger than a warp's buffer
};

// The decoder's error record: {0, -, -} or {kind, block, code}.
enum DecodeError : uint32_t { kDecOk = 0, kDecBad = 1, kDecShort = 2 };

// Validates the chunk against the frame (the reference's checks and texts)
// and fills the block table. SF_OK, or an error code with t_last_error set.
int plan_chunk(const uint8_t *data, size_t nbytes, const char *algorithm, unsigned bit_depth,
               size_t height, size_t width, size_t out_bytes, ChunkPlan *plan);

// Decodes the table's blocks of d_payload into d_frame (16-byte aligned).
// d_scratch (plan.frame_bytes) is needed when plan.scratch is set; d_status
// (3 words, zeroed by the caller) receives the first error seen; d_next (a
// word, zeroed by the caller) hands the blocks out to the warps.
cudaError_t launch_decode(const uint8_t *d_payload, const DecodeBlock *d_blocks, size_t nblocks,
                          unsigned element, uint8_t *d_frame, uint8_t *d_scratch,
                          uint32_t *d_status, uint32_t *d_next, cudaStream_t stream);

// The reference's exception text for a decoder error record.
std::string decode_error_text(const ChunkPlan &plan, const uint32_t status[3]);

extern thread_local std::string t_last_error;

}  // namespace sf
