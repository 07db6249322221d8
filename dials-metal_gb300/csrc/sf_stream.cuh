// Internal interface of the streaming threshold (sf_stream.cu).
//
// The float decision of the dispersion test. With exact n, S (integers) and
// Q~ = the float sum of the window's p^2 (13 roundings of non-negative terms
// at most, so Q~ = Q (1 + e), |e| <= 13 u, u = 2^-24), the reference's test
// at gain 1 and integral sigma_b is A > RN(X) with A = nQ - S(S + n - 1)
// exact and X = S sigma_b r_n (the reference's double r_n). Writing
// c = n - 1 + sigma_b r_n, A - X = nQ - S(S + c). Tables per n give floats
// nf_hi >= n (1 + 2^-14), nf_lo <= n (1 - 2^-14) and c_lo <= c <= c_hi.
//   RN(nf_hi Q~) <= RN(S~ RN(S~ + c_lo))     =>  nQ <= S(S + c): not signal
//   RN(nf_lo Q~) >= RN(RN(1.0001 RN(S~ RN(S~ + c_hi))) + 2)
//                                            =>  nQ >= S(S + c) + 1: signal
// (the 2^-14 and 1.0001 margins exceed the few-u float errors by orders of
// magnitude). Anything else is decided exactly. The packed sums (count above
// a 27-, 26- or 25-bit sum for K = 2, 3, 4) hold while every valid pixel is
// below 2^bits / n_max, which also keeps nQ < 2^53 and S^2 < 2^52, where the
// reference's double left side is exactly A.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sf_common.cuh"

namespace sf {

// Counter words at the start of the stream workspace.
enum {
  kCtrTotal = 0,  // signal pixels found
  kCtrCand,       // candidates found
  kCtrWide,       // runs handed to the 64-bit path
  kCtrCount = 8
};

// Strips of 240 output columns (one warp each) by runs of rows: as many runs
// as fill the GPU once (3 blocks of 4 warps on each of 152 SMs), each at least
// 16 rows.
struct SegGeometry {
  int nstrips, nruns, run_rows;
};
inline SegGeometry seg_geometry(int h, int w) {
  SegGeometry g;
  g.nstrips = (w + 239) / 240;
  const int target = 1800;
  int nruns = (target + g.nstrips - 1) / g.nstrips;
  g.run_rows = (h + nruns - 1) / nruns;
  if (g.run_rows < 16)
    g.run_rows = 16;
  g.nruns = (h + g.run_rows - 1) / g.run_rows;
  return g;
}

struct StreamTables {
  uint32_t narrow_max;  // valid pixels at or above this take the 64-bit path
  float nf_hi[kMaxN0 + 1], nf_lo[kMaxN0 + 1], c_lo[kMaxN0 + 1], c_hi[kMaxN0 + 1];
};

struct StreamBuffers {
  uint32_t *bits;         // final strong mask (output)
  uint32_t *scr1;         // eroded mask
  uint32_t *prefix;       // per-word exclusive popcount prefix (maybe output)
  uint32_t *cand;         // candidate pixel indices
  uint32_t cand_cap;
  uint32_t *counters;     // kCtrCount words
  uint4 *wide;            // handed-over runs
  uint32_t *block_sums;   // per-block sums of the ordering kernel
  sf_signal_pixel *staging;
  sf_signal_pixel *out;   // ascending list (output)
  uint32_t capacity;
  uint32_t *count_out;    // the caller's count word
};

inline int stream_units(int h, int w) {
  const SegGeometry g = seg_geometry(h, w);
  return g.nstrips * g.nruns;
}


void make_stream_tables(const LaunchParams &P, StreamTables *T);

cudaError_t launch_stream(const uint32_t *image, int h, int w, const LaunchParams &P,
                          const StreamBuffers &b, cudaStream_t stream);

} // namespace sf
