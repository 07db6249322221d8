// Internal interface of the streaming threshold (sf_stream.cu): 32-bit
// frames, dispersion_extended, gain 1 and integral sigmas, one frame or a
// batch of same-shaped frames per launch sequence.
//
// The stage-0 decision from exact 32-bit window sums. With gain 1 and an
// integral sigma_b the reference's test (src/spots/dext.cc:99-109) is
// A > RN(X), A = nQ - S(S + n - 1) exact in double and X = S sigma_b r_n
// (r_n the reference's double sqrt(2 (n - 1))). Writing c = n - 1 +
// sigma_b r_n, A - X = nQ - S(S + c). Per window count n the host gives two
// integers in 2^-8 units, clo <= 2^8 c <= chi (from the 2^-20 brackets of
// r_n), and nk = 2^8 n (0 when n cannot be tested):
//   2^8 n Q <= S (2^8 S + clo)           =>  A <= X: not signal
//   2^8 n Q >= S (2^8 S + chi) + 2^9     =>  A >= X + 2 > RN(X): signal
// both exact in 64-bit integers. The thin band between goes to the exact
// decision of sf_common.cuh. The packed sums (the window's masked-pixel count
// above a 27-, 26- or 25-bit sum for K = 2, 3, 4) and the 32-bit sum of
// squares hold while every valid pixel is below narrow_max; a run holding a
// larger valid pixel is handed to a 64-bit path.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "sf_common.cuh"

namespace sf {

// The current device's SM count (152 until a device answers).
int device_sms();

// Frames one launch sequence takes.
constexpr int kMaxBatch = 64;

// A launch's frames and each one's shape. Frames of one launch may differ
// in shape on the kernel-3,3 lattice path (launch_stream, launch_stream16:
// every buffer is laid out for the largest, h x w, and each frame uses its
// own rows of it); the other paths take frames of one shape.
struct FramePtrs {
  const uint32_t *image[kMaxBatch];
  int h[kMaxBatch], w[kMaxBatch];
};

// Mask words of frame f (its own rows of ceil(w / 32) words).
__host__ __device__ inline size_t frame_words(const FramePtrs &F, int f) {
  return (size_t)((F.w[f] + 31) >> 5) * (size_t)F.h[f];
}

// Counter words: the batch's own first, then kCtrCount per frame.
enum {
  kCtrWide = 0,   // batch: runs handed to the 64-bit path
  kCtrTiles = 1,  // batch: tiles listed for the exact check (kernel 3,3)
  kCtrTiles2 = 2, // batch: tiles with a candidate left after it (stage 2's list)
  kCtrFault = 3,  // batch: a bounded device wait ran out (the launch's lists are void)
  kCtrBatch = 4,  // first frame's counters
  kCtrCand = 0,   // frame: candidates (set bits of the candidate mask)
  kCtrWideFrame = 1,  // frame: a valid pixel may be too large for 32-bit stage-2 sums
  kCtrCount = 4
};
inline size_t counter_words(int nframes) { return kCtrBatch + (size_t)nframes * kCtrCount; }

// A frame's signal count when its launch met a device fault (kCtrFault):
// no list, whatever the capacity.
constexpr uint32_t kCountFault = 0xFFFFFFFEu;

// Strips of 240 output columns (one warp each) by runs of run_rows rows.
struct SegGeometry {
  int nstrips, nruns, run_rows;
};
// run_rows 0 picks runs that fill `slots` warps once.
SegGeometry seg_geometry(int h, int w, int nframes, int run_rows, int slots);
constexpr int kMinRunRows = 16;

struct StreamTables {
  uint32_t narrow_max;  // valid pixels at or above this take the 64-bit path
  uint32_t nk[kMaxN0 + 1], clo[kMaxN0 + 1], chi[kMaxN0 + 1];
};

struct StreamBuffers {
  uint32_t *bits;          // final strong masks (output), frame f at bits + f * words
  uint32_t *scr1;          // eroded masks, same layout
  uint32_t *amb;           // ambiguous stage-0 windows, same layout (kernel 3,3: see lattice_tiles)
  uint32_t *prefix;        // per-word list positions (output) or null
  size_t words;            // mask words per frame
  uint32_t *cand;          // ascending candidate indices, frame f at cand + f * cand_cap
  uint2 *res;              // stage-2 result per candidate, same layout
  uint32_t cand_cap;
  uint32_t *counters;      // counter_words(nframes)
  uint4 *wide;             // handed-over runs, two uint4 each
  uint32_t *block_sums;    // per-block sums of the scan kernels
  uint32_t capacity;
  sf_signal_pixel *out;    // ascending lists (output), frame f at out + f * out_stride
  size_t out_stride;
  uint32_t *count_out;     // one count per frame
};

// Wide-list entries a batch may need (every run hands over at most once).
size_t stream_wide_entries(int h, int w, int nframes);
// Blocks of the ordering kernel (the size of block_sums).
int stream_order_blocks();

void make_stream_tables(const LaunchParams &P, StreamTables *T);

// The run length the default geometry picks for a batch (the tuner's start).
int stream_default_run_rows(const LaunchParams &P, int h, int w, int nframes);

// Events recorded on the stream between the kernel groups when profiling.
struct StreamMarks {
  cudaEvent_t start, stage01, stage2, order;
};

// The lattice pass for kernel 3,3 (sf_lattice.cu): strips of 360 output
// columns (one warp each) by runs of run_rows rows, a multiple of 3.
struct LatticeGeometry {
  int nstrips, nruns, run_rows;
};
// run_rows 0 picks runs that fill the resident warps once.
LatticeGeometry lattice_geometry(int h, int w, int nframes, int run_rows);
// Tiles of the exact check a frame has. For kernel 3,3 StreamBuffers::amb
// holds words + 2 lattice_tiles words a frame: the candidate mask's per-word
// list positions, the tile list, and the list of tiles left for stage 2.
size_t lattice_tiles(int h, int w);
// Stage 2 for kernel 3,3 on the listed tiles, after launch_lattice and
// mask_prefix into b.amb: the candidate list and the results (b.cand, b.res).
cudaError_t launch_lattice_stage2(const FramePtrs &frames, int nframes, int h, int w, int vec,
                                  int pixel_bytes, const LaunchParams &P, const StreamBuffers &b,
                                  cudaStream_t stream);
// Stage 0 and the erosion for kernel 3,3: the lattice bound, then the exact
// check of its candidates; writes b.bits as the first pass of launch_stream
// does (vec: the frames allow 16-byte loads). b.scr1 is not used: stage 2
// takes the eroded mask as b.bits plus the masked pixels.
// pixel_bytes 4 (32-bit frames) or 2 (16-bit frames: 4 | w, 8-byte aligned).
cudaError_t launch_lattice(const FramePtrs &frames, int nframes, int h, int w, int vec,
                           int pixel_bytes, const LaunchParams &P, const StreamTables &T,
                           const StreamBuffers &b, int run_rows, cudaStream_t stream);

// 16-bit frames, kernel 3,3, dispersion_extended (any gain and sigmas; the
// tests are the reference's float ones): the lattice path of launch_stream.
// The frames' width must be a multiple of 4 and each frame 8-byte aligned.
cudaError_t launch_stream16(const FramePtrs &frames, int nframes, int h, int w,
                            const LaunchParams &P, const StreamBuffers &b, int run_rows,
                            cudaStream_t stream, const StreamMarks *marks = nullptr);

// run_rows 0: the default geometry. marks may be null.
cudaError_t launch_stream(const FramePtrs &frames, int nframes, int h, int w,
                          const LaunchParams &P, const StreamBuffers &b, int run_rows,
                          cudaStream_t stream, const StreamMarks *marks = nullptr);

} // namespace sf
