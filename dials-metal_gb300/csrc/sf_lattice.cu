// Stage 0 and the erosion of the streaming threshold for the reference's own
// window (kernel 3,3: 7 x 7 stage-0 windows, erosion by 2), in two kernels:
//
//   lat_stage01  stage 0 on a lattice of every third row and every third
//                column only, and the erosion of that lattice: an upper bound
//                of the eroded mask, written as the candidate mask
//   lat_verify   the exact stage 0 and erosion on the 8 x 28 tiles that hold
//                a candidate of the bound; the candidates that fail leave the
//                mask, which is then the reference's candidate mask
//
// The reference's eroded mask (stage 1's signal after the erosion, which
// stage 2 keeps out of each background) is the candidate mask with the
// masked pixels added, and stage 2 reads it so: the candidate mask's bits
// and its staged pixels' masked values. No separate eroded mask is written.
//
// Why the bound holds. The erosion (src/spots/dext.cc:117-142) keeps a valid
// pixel only if every in-frame pixel of its 5 x 5 neighbourhood is signal or
// masked after stage 0. ANDing over only the lattice pixels of the
// neighbourhood can keep more pixels, never fewer. Every 5 x 5 neighbourhood
// holds 1 to 4 lattice pixels, and next to a masked band or the frame's edge
// a valid pixel still sees a 3 x 3 block of in-frame valid pixels, so a
// lattice pixel; the bound passes about 1.7 times the exact candidates, all in
// and around spots.
//
// The lattice decisions are an upper bound too: a window counts as signal
// when the lower of the two integer bounds of sf_stream.cuh says it may be,
// and when its sums may not be exact. Valid pixels are summed saturated at
// kLatCap (2^15 - 1), so every packed sum is exact for the saturated values;
// a window whose saturated sum S is below kLatCap - 1 holds no saturated
// pixel, its sum of squares is at most S^2 < 2^30, and its decision is that
// of the reference. A window with a larger S is taken as signal, and the tile
// check decides it exactly.
//
// The tile check decides only the stage-0 windows within 2 of a candidate
// (the only ones whose decision can clear one), about a fifth of a tile's,
// spread over the warp's lanes. Its 18 x 38 pixels cover the stage-2 window
// (11 x 11) of every candidate of the tile, so it is also where a frame is
// marked for the 64-bit stage 2: a tile holding a valid pixel at or above
// narrow_max marks its frame.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include <cudaTypedefs.h>

#include "sf_common.cuh"
#include "sf_stream.cuh"
#include "sf_tma.cuh"

namespace sf {
namespace {

constexpr int kLatK = 3;                    // stage-0 half-width
constexpr int kLatN0 = 49;                  // pixels of a stage-0 window
constexpr int kLatCols = 12;                // columns a lane owns
constexpr int kLatOutLanes = 30;            // lanes 1-30 write; lanes 0 and 31 are their halos
constexpr int kLatOut = kLatCols * kLatOutLanes;  // 360 output columns a warp
constexpr int kLatWarps = 4;                // warps a block
constexpr int kLatOcc = 5;                  // blocks an SM the kernel is built for
constexpr uint32_t kLatPS = 26;             // masked count above a 26-bit sum
constexpr uint32_t kLatMask = (1u << kLatPS) - 1u;
constexpr uint32_t kLatCap = 32767;         // valid pixels saturate here
constexpr int kDec = 8;                     // fixed-point bits of clo / chi

static_assert(kLatOut % 24 == 0, "lane pairs write whole bytes");

// Division of 32-bit numerators by a divisor fixed for a launch (tile
// counts), by one multiply-high and shifts: the round-up method of
// Granlund & Montgomery, "Division by invariant integers using
// multiplication" (PLDI 1994), with its add-and-shift step for multipliers of
// 33 bits. Exact for every numerator and divisor below 2^32.
struct FastDiv {
  uint32_t d, m, s1, s2;
};

// Marks a tile of stage 2's list whose candidates all failed the exact check.
constexpr uint32_t kNoTile = 0xFFFFFFFFu;

FastDiv make_fastdiv(uint32_t d) {
  int l = 0;
  while ((1ull << l) < d)
    l++;
  FastDiv f;
  f.d = d;
  f.m = (uint32_t)(((((unsigned long long)1 << l) - d) << 32) / d + 1);
  f.s1 = l < 1 ? (uint32_t)l : 1u;
  f.s2 = l > 1 ? (uint32_t)(l - 1) : 0u;
  return f;
}

__device__ __forceinline__ uint32_t fast_div(uint32_t n, const FastDiv &f) {
  const uint32_t t = __umulhi(n, f.m);
  return (t + ((n - t) >> f.s1)) >> f.s2;
}


static_assert(kLatN0 * kLatCap < (1u << kLatPS), "saturated sums stay below the count field");

// Where each frame's share of a launch's warps (lat_stage01: strips x runs)
// or tile groups (lat_tiles: tile rows x groups of 32 tiles) starts, and how
// many make one of its rows: every frame of a batch, mixed shapes or not,
// gets exactly its own.
struct FrameSpans {
  int start[kMaxBatch + 1];
  FastDiv by_row[kMaxBatch];
};

// The frame whose span holds item g (start[f] <= g < start[f + 1]); g below
// start[nframes].
__device__ __forceinline__ int span_frame(const FrameSpans &S, int nframes, int g) {
  int lo = 0, hi = nframes;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (S.start[mid] <= g)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// The 12 bound bits of a lane from the lattice bits b0-b4 at its columns
// -1, 2, 5, 8 and 11 (b0 is the lane before's column 11): column c keeps the
// lattice columns within 2 of it.
__host__ __device__ constexpr uint32_t lat_bound12(uint32_t b) {
  const uint32_t b0 = b & 1u, b1 = (b >> 1) & 1u, b2 = (b >> 2) & 1u, b3 = (b >> 3) & 1u,
                 b4 = (b >> 4) & 1u;
  const uint32_t a = b0 & b1, d = b1 & b2, e = b2 & b3, g = b3 & b4;
  return a * 0x003u | b1 << 2 | d * 0x018u | b2 << 5 | e * 0x0C0u | b3 << 8 | g * 0x600u |
         b4 << 11;
}

__device__ __forceinline__ void lat_load(const uint32_t *__restrict__ image, int height, int width,
                                         bool interior, int cx, int p, uint32_t v[kLatCols]) {
  if (p < 0 || p >= height) {
#pragma unroll
    for (int i = 0; i < kLatCols; i++)
      v[i] = 0xFFFFFFFFu;
    return;
  }
  const uint32_t *row = image + (size_t)p * width + cx;
  if (interior) {
#pragma unroll
    for (int f = 0; f < kLatCols / 4; f++) {
      const uint4 t = __ldg(reinterpret_cast<const uint4 *>(row) + f);
      v[4 * f] = t.x, v[4 * f + 1] = t.y, v[4 * f + 2] = t.z, v[4 * f + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < kLatCols; i++) {
      const int gx = cx + i;
      v[i] = (gx >= 0 && gx < width) ? __ldg(row + i) : 0xFFFFFFFFu;
    }
  }
}

// One pixel row of a lane: its 12 pixels packed (masked as a lone count bit
// whose square wraps to 0, valid saturated at kLatCap), the row sums of 7
// columns at the lattice columns 2, 5, 8, 11, and the masked bits of the 12
// columns. The windows reach one column into the lane before (its column 11,
// by a shuffle) and three into the lane after (its first triple, likewise):
// lanes 0 and 31 hold the halo columns of the warp's 30 writing lanes.
// 16-bit frames (Pix = uint16_t) are summed as the reference sums them: in
// 32 bits, the sum of squares modulo 2^32 (src/spots/dext.hh:31-33); their
// pixels need no saturation (49 of them sum below 2^22).
template <typename Pix>
__device__ __forceinline__ void lat_row(const uint32_t v[kLatCols], int lane, uint32_t hn[4],
                                        uint32_t hq[4], uint32_t *m12) {
  constexpr bool k16 = sizeof(Pix) == 2;
  uint32_t ns[kLatCols], q[kLatCols];
#pragma unroll
  for (int i = 0; i < kLatCols; i++) {
    if (k16)
      ns[i] = v[i] >= 0xFFFEu ? (1u << kLatPS) : v[i];
    else
      ns[i] = v[i] >= 0xFFFFFFFEu ? (1u << kLatPS) : min(v[i], kLatCap);
    q[i] = ns[i] * ns[i];
  }
  // Triples of columns [3a, 3a + 2], then the 7-column windows.
  uint32_t gn[4], gq[4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    gn[a] = ns[3 * a] + ns[3 * a + 1] + ns[3 * a + 2];
    gq[a] = q[3 * a] + q[3 * a + 1] + q[3 * a + 2];
  }
  const uint32_t ln = __shfl_sync(0xffffffffu, ns[kLatCols - 1], (lane + 31) & 31);
  const uint32_t lq = __shfl_sync(0xffffffffu, q[kLatCols - 1], (lane + 31) & 31);
  const uint32_t rn = __shfl_sync(0xffffffffu, gn[0], (lane + 1) & 31);
  const uint32_t rq = __shfl_sync(0xffffffffu, gq[0], (lane + 1) & 31);
  hn[0] = ln + gn[0] + gn[1];
  hq[0] = lq + gq[0] + gq[1];
  hn[1] = ns[2] + gn[1] + gn[2];
  hq[1] = q[2] + gq[1] + gq[2];
  hn[2] = ns[5] + gn[2] + gn[3];
  hq[2] = q[5] + gq[2] + gq[3];
  hn[3] = ns[8] + gn[3] + rn;
  hq[3] = q[8] + gq[3] + rq;
  // A valid packed 32-bit-frame pixel is below 2^15, so shifting it right by
  // 26 - c (c <= 11) leaves nothing: the shifted words add up to the masked
  // bits. A 16-bit pixel can reach 2^16, so its count bit is isolated first.
  uint32_t m = 0;
#pragma unroll
  for (int c = 0; c < kLatCols; c++)
    m += k16 ? (ns[c] >> kLatPS) << c : ns[c] >> (kLatPS - c);
  *m12 = m;
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
// One piece of 4 pixels: 16 bytes of a 32-bit frame, 8 of a 16-bit one.
template <typename Pix> __device__ __forceinline__ void cp_async_piece(void *dst, const void *src) {
  if (sizeof(Pix) == 4)
    cp_async16(dst, src);
  else
    cp_async8(dst, src);
}
template <typename Pix> __device__ __forceinline__ void fill_piece_masked(void *dst) {
  if (sizeof(Pix) == 4)
    *reinterpret_cast<uint4 *>(dst) = make_uint4(~0u, ~0u, ~0u, ~0u);
  else
    *reinterpret_cast<uint2 *>(dst) = make_uint2(~0u, ~0u);
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// The ring variant (kRing: 4 | width and 16-byte aligned frames) stages each
// warp's pixel rows in shared memory by cp.async, kRingSlots - 1 rows ahead:
// a row is the 96 16-byte pieces from column X - 12 (X the strip's first
// output column) that the lanes read, 12 columns a lane. The other variant
// loads each lane's 12 columns straight from the frame, a row ahead.
//
// A piece is 4 pixels: 16 bytes of a 32-bit frame, 8 of a 16-bit one (whose
// rows, with 4 | width, start 8-byte aligned). Both fetch 96 pieces from
// column X - 12, and lane l reads its 12 pixels from column 12 l of the slot.
constexpr int kRingSlots = 4;
constexpr int kRingPieces = 96;   // pieces fetched a row: 3 a lane
constexpr int kRingStride = 384;  // pixels a slot
template <typename Pix>
constexpr size_t ring_bytes() {
  return (size_t)kLatWarps * kRingSlots * kRingStride * sizeof(Pix);
}

template <int kOcc, bool kRing, typename Pix>
__global__ void __launch_bounds__(kLatWarps * 32, kOcc)
lat_stage01(const __grid_constant__ FramePtrs F, int nframes, int vec,
            const __grid_constant__ FrameSpans S, int run_rows,
            const __grid_constant__ StreamTables T,
            const __grid_constant__ LaunchParams P, uint8_t *__restrict__ final_bytes,
            size_t mask_bytes) {
  constexpr bool k16 = sizeof(Pix) == 2;
  static_assert(!k16 || kRing, "16-bit frames take the ring variant only");
  extern __shared__ __align__(16) unsigned char lat_ring_raw[];
  Pix *lat_ring = reinterpret_cast<Pix *>(lat_ring_raw);
  // Lower-bound constants by masked count m (window count 49 - m).
  __shared__ uint2 tab[kLatN0 + 1];
  __shared__ uint16_t lut[32];
  for (int m = threadIdx.x; m <= kLatN0; m += blockDim.x)
    tab[m] = make_uint2(T.nk[kLatN0 - m], T.clo[kLatN0 - m]);
  if (threadIdx.x < 32)
    lut[threadIdx.x] = (uint16_t)lat_bound12(threadIdx.x);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gw = blockIdx.x * kLatWarps + warp;
  if (gw >= S.start[nframes])
    return;  // whole warp
  // This warp's frame, strip and run (each frame has its own strips x runs).
  const int f = span_frame(S, nframes, gw);
  const uint32_t local = (uint32_t)(gw - S.start[f]);
  const int ry = (int)fast_div(local, S.by_row[f]);
  const int sx = (int)(local - (uint32_t)ry * S.by_row[f].d);
  const int height = F.h[f], width = F.w[f];
  const Pix *image = reinterpret_cast<const Pix *>(F.image[f]);
  const int bytes_per_row = ((width + 31) >> 5) * 4;
  uint8_t *fin = final_bytes + (size_t)f * mask_bytes;
  // Lane l holds columns X + 12 (l - 1) .. + 11: lanes 1-30 the strip's
  // 360, lane 0 the 12 before it, lane 31 the 12 after it.
  const int cx = kLatOut * sx + kLatCols * (lane - 1);
  const bool interior = vec && cx >= 0 && cx + kLatCols <= width;
  // This lane's first mask byte (lane pairs 1-2, 3-4, .. share three
  // bytes), and the bits of its columns inside the frame.
  const int pair_byte = (kLatOut * sx + 24 * ((lane - 1) >> 1)) >> 3;
  const bool writer = lane >= 1 && lane <= kLatOutLanes;
  const bool first_of_pair = (lane & 1) != 0;
  const uint32_t inside12 =
      (cx < 0 || cx >= width) ? 0u
                              : (cx + kLatCols <= width ? 0xFFFu : ((1u << (width - cx)) - 1u));
  const int ra = ry * run_rows;
  const int rb = min(height, ra + run_rows);
  const int ja = ra / 3;
  const int ntrip = (rb - ra + 2) / 3;

  // U = h(last row of triple t-2) + T(t-1) per lattice column; hl = the
  // last row of the previous triple.
  uint32_t Un[4], Uq[4], hln[4], hlq[4];
#pragma unroll
  for (int a = 0; a < 4; a++)
    Un[a] = Uq[a] = hln[a] = hlq[a] = 0u;
  uint32_t mprev[3] = {0u, 0u, 0u}, bprev = 0u, cmprev = 0u;

  // Pixel rows [pbeg, pend) of the run.
  const int pbeg = 3 * (ja - 2), pend = 3 * (ja + ntrip + 1);
  Pix *ring = lat_ring + (size_t)warp * kRingSlots * kRingStride;
  // The ring's pieces of this lane: l, l + 32, l + 64 (a warp's copy
  // instruction covers 128 contiguous pixels), and whether each lies in the
  // frame.
  const int X = kLatOut * sx;
  const int x0 = X - kLatCols + 4 * lane;
  bool pin[3];
#pragma unroll
  for (int i = 0; i < 3; i++)
    pin[i] = x0 + 128 * i >= 0 && x0 + 128 * i + 4 <= width;
  auto fetch = [&](int p) {
    Pix *dst = ring + ((p - pbeg) % kRingSlots) * kRingStride + 4 * lane;
    const bool rowin = p >= 0 && p < height && p < pend;
    const Pix *src = image + (size_t)(rowin ? p : 0) * width + x0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      if (rowin && pin[i])
        cp_async_piece<Pix>(dst + 128 * i, src + 128 * i);
      else
        fill_piece_masked<Pix>(dst + 128 * i);
    }
  };
  if (kRing) {
#pragma unroll
    for (int i = 0; i < kRingSlots - 1; i++) {
      fetch(pbeg + i);
      cp_async_commit();
    }
  }

  uint32_t v[kLatCols];
  if constexpr (!kRing)
    lat_load(reinterpret_cast<const uint32_t *>(image), height, width, interior, cx, pbeg, v);
  for (int t = 0; t < ntrip + 3; t++) {
    const int p0 = 3 * (ja - 2 + t);
    uint32_t Tn[4], Tq[4], mcur[3], cm = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int p = p0 + k;
      uint32_t nxt[kLatCols];
      if (kRing) {
        // Row p + kRingSlots - 1 goes out; row p has landed.
        __syncwarp();
        fetch(p + kRingSlots - 1);
        cp_async_commit();
        cp_async_wait<kRingSlots - 1>();
        __syncwarp();
        const Pix *slot = ring + ((p - pbeg) % kRingSlots) * kRingStride;
        if constexpr (k16) {
          const uint2 *src = reinterpret_cast<const uint2 *>(slot + kLatCols * lane);
#pragma unroll
          for (int i = 0; i < kLatCols / 4; i++) {
            const uint2 x = src[i];
            v[4 * i] = x.x & 0xFFFFu, v[4 * i + 1] = x.x >> 16;
            v[4 * i + 2] = x.y & 0xFFFFu, v[4 * i + 3] = x.y >> 16;
          }
        } else {
          const uint4 *src = reinterpret_cast<const uint4 *>(slot) + 3 * lane;
#pragma unroll
          for (int i = 0; i < kLatCols / 4; i++) {
            const uint4 x = src[i];
            v[4 * i] = x.x, v[4 * i + 1] = x.y, v[4 * i + 2] = x.z, v[4 * i + 3] = x.w;
          }
        }
      } else if (k < 2 || t + 1 < ntrip + 3) {
        // The next row's loads go out before this row's arithmetic.
        lat_load(reinterpret_cast<const uint32_t *>(image), height, width, interior, cx,
                 p + 1, nxt);
      }
      uint32_t hn[4], hq[4];
      lat_row<Pix>(v, lane, hn, hq, &mcur[k]);
      if (!kRing) {
#pragma unroll
        for (int i = 0; i < kLatCols; i++)
          v[i] = nxt[i];
      }
#pragma unroll
      for (int a = 0; a < 4; a++) {
        Tn[a] = k == 0 ? hn[a] : Tn[a] + hn[a];
        Tq[a] = k == 0 ? hq[a] : Tq[a] + hq[a];
      }
      if (k == 2) {
        // Masked centres of this row's lattice columns 2, 5, 8, 11: the
        // lattice row the next triple decides.
        const uint32_t m12 = mcur[2];
        cm = ((m12 >> 2) & 1u) | ((m12 >> 4) & 2u) | ((m12 >> 6) & 4u) | ((m12 >> 8) & 8u);
#pragma unroll
        for (int a = 0; a < 4; a++) {
          // Window rows p0 - 4 .. p0 + 2, centred on the previous triple's
          // last row (a lattice row).
          const uint32_t Wn = Un[a] + Tn[a], Wq = Uq[a] + Tq[a];
          Un[a] = hln[a] + Tn[a];
          Uq[a] = hlq[a] + Tq[a];
          hln[a] = hn[a];
          hlq[a] = hq[a];
          Tn[a] = Wn;
          Tq[a] = Wq;
        }
      }
    }
    if (t < 2) {
      cmprev = cm;
#pragma unroll
      for (int k = 0; k < 3; k++)
        mprev[k] = mcur[k];
      continue;  // warp-uniform: the windows are not yet whole
    }
    // Lattice row p0 - 1: four decisions by the lower bound (sf_stream.cuh),
    // windows whose sums may be inexact taken as signal, masked centres set.
    uint32_t b4 = cmprev;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const uint32_t W = Tn[a];
      const uint32_t m = min(W >> kLatPS, (uint32_t)kLatN0);  // 49 pixels: m <= 49
      const uint32_t S = W & kLatMask;
      bool sig;
      if constexpr (k16) {
        // The reference's float test, exactly (sf_common.cuh stage0_u16).
        sig = stage0_u16((uint32_t)kLatN0 - m, S, Tq[a], P);
      } else {
        const uint2 c = tab[m];
        const unsigned long long L = (unsigned long long)Tq[a] * c.x;
        const unsigned long long Rr = (unsigned long long)S * ((S << kDec) + c.y);
        sig = L > Rr || S >= kLatCap - 1u;
      }
      b4 |= sig ? 1u << a : 0u;
    }
    // The bound bits at columns -1 (the lane before's 11), 2, 5, 8, 11.
    const uint32_t b5 = b4 << 1 | (__shfl_sync(0xffffffffu, b4, (lane + 31) & 31) >> 3 & 1u);
    if (t >= 3) {
      // The previous triple's rows p0 - 3 .. p0 - 1: the first two see the
      // lattice rows p0 - 4 and p0 - 1, the last only p0 - 1.
      const uint32_t bd01 = lut[bprev & b5], bd2 = lut[b5];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const int r = p0 - 3 + k;
        const uint32_t bd = k < 2 ? bd01 : bd2;
        const uint32_t mk = mprev[k];
        const uint32_t c12 = bd & ~mk & inside12;
        // Lane pairs: the first lane (odd) writes the pair's first two bytes,
        // the second the third.
        const uint32_t odd = __shfl_down_sync(0xffffffffu, c12, 1);
        if (writer && r < rb) {
          const size_t at = (size_t)r * bytes_per_row;
          if (first_of_pair) {
            if (pair_byte < bytes_per_row)
              fin[at + pair_byte] = (uint8_t)c12;
            if (pair_byte + 1 < bytes_per_row)
              fin[at + pair_byte + 1] = (uint8_t)((c12 >> 8) | (odd & 0xFu) << 4);
          } else if (pair_byte + 2 < bytes_per_row) {
            fin[at + pair_byte + 2] = (uint8_t)(c12 >> 4);
          }
        }
      }
    }
    bprev = b5;
    cmprev = cm;
#pragma unroll
    for (int k = 0; k < 3; k++)
      mprev[k] = mcur[k];
  }
  if (kRing)
    cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// The exact check of the bound's candidates, on tiles of 8 rows x 28 columns.
//
//   lat_tiles   lists the tiles that hold a candidate (any order)
//   lat_verify  one warp per listed tile, persistent: the tile's 12 x 32
//               stage-0 windows (rows r0 - 2 .., columns c0 - 2 .., lane =
//               column) from its 18 x 38 pixels, the erosion of its 8 x 28
//               pixels, and the candidates that fail cleared from both masks
//
// A warp copies the next tile's pixels into shared memory (cp.async, 16-byte
// pieces where the frame allows) while it checks the current one, so the
// loads' latency is hidden behind the arithmetic. Column sums of 7 rows go to
// shared memory; then only the stage-0 windows within 2 of a candidate (the
// only ones that can clear one, about a fifth of the tile's) are decided,
// spread over the lanes: the two bounds of sf_stream.cuh, and the reference's
// sequence between them (sf_common.cuh). Tiles share mask words, so the
// clearing is an atomic AND; each candidate belongs to one tile, so the order
// does not matter. A tile's 18 x 38 pixels cover the stage-2 window (11 x 11)
// of each of its candidates, so a tile holding a valid pixel at or above
// narrow_max marks its frame for the 64-bit stage 2.
// ---------------------------------------------------------------------------
constexpr int kVerRows = 8;                  // output rows of a tile
constexpr int kVerTW = 28;                   // output columns of a tile
constexpr int kVerPR = kVerRows + 10;        // pixel rows
constexpr int kVerDR = kVerRows + 4;         // stage-0 rows
constexpr int kVerPC = 38;                   // pixel columns
constexpr int kVerPW = 44;                   // staged columns: 11 16-byte pieces
constexpr int kVerWarps = 4;
constexpr int kVerOcc = 6;                   // exact-check blocks an SM (a pixel buffer a warp)
constexpr int kS2Occ = 5;                    // stage-2 blocks an SM (two pixel buffers a warp)

__host__ __device__ inline int ver_ntx(int w) { return (w + kVerTW - 1) / kVerTW; }
__host__ __device__ inline int ver_nty(int h) { return (h + kVerRows - 1) / kVerRows; }

// Staged columns a pixel row (whole 16-byte pieces covering the 38 needed
// from a 16-byte boundary) and that boundary's alignment, in pixels: a TMA
// box row must be a multiple of 16 bytes and start on one.
template <typename Pix> struct VerPix;
template <> struct VerPix<uint32_t> {
  static constexpr int kPW = kVerPW, kAlign = 4;
};
template <> struct VerPix<uint16_t> {
  static constexpr int kPW = 48, kAlign = 8;
};

// One staged tile: 18 pixel rows (r0 - 5 .. r0 + 12) of kPW pixels from the
// aligned column xs, dense, as a TMA box lands in shared memory (128-byte
// aligned, the box load's destination rule).
template <typename Pix> struct alignas(128) TileBuf {
  Pix px[kVerPR][VerPix<Pix>::kPW];
};

template <typename Pix> struct alignas(128) VerWarp {
  TileBuf<Pix> pix[1];                   // staged pixels (the next tile's load goes out
                                         // once the current one's are read)
  uint64_t bar[1];                       // its TMA mbarrier
  uint32_t cw[2][kVerRows][2];           // the tile's candidate words, two tiles (s)
  uint2 vs[kVerDR][kVerPC + 2];          // column sums of 7 rows
  uint32_t msk[kVerPC + 2];              // masked pixels by row, a word a column
};

// The frames' 2-D tensor maps, boxes of one tile (kPW x 18 pixels), for the
// TMA staging of the exact check and stage 2.
struct TileMaps {
  CUtensorMap map[kMaxBatch];
};

template <typename Pix> __device__ __forceinline__ bool is_masked_px(uint32_t v) {
  return sizeof(Pix) == 2 ? v >= 0xFFFEu : v >= 0xFFFFFFFEu;
}

// The reference's decision for one window from exact sums, out of line: the
// callers reach it only between the two bounds.
__device__ __noinline__ bool lat_exact(uint32_t n, uint32_t S, uint32_t Q, const LaunchParams &P) {
  return stage0_u32(n, S, Q, P, P.root_lo, P.root_hi);
}

// The stage-0 bit (signal or masked; off the frame counts as set) of the
// window whose top-left staged pixel is (row, col) of a staged tile, with
// 64-bit sums, for tiles holding a pixel too large for the 32-bit ones. The
// staged tile holds pixels off the frame as masked, so they are skipped as
// the reference's clipped window skips them.
__device__ __noinline__ bool lat_wide(const uint32_t (*px)[kVerPW], int row, int col,
                                      const LaunchParams &P) {
  if (px[row + kLatK][col + kLatK] >= 0xFFFFFFFEu)
    return true;
  uint32_t n = 0;
  unsigned long long S = 0, Q = 0;
  for (int dy = 0; dy <= 2 * kLatK; dy++) {
#pragma unroll
    for (int dx = 0; dx <= 2 * kLatK; dx++) {
      const uint32_t v = px[row + dy][col + dx];
      if (v < 0xFFFFFFFEu) {
        n++;
        S += v;
        Q += (unsigned long long)v * v;
      }
    }
  }
  return stage0_u32(n, S, Q, P, P.root_lo, P.root_hi);
}

// Tiles of a tile row come in groups of 32 consecutive ones: 32 tiles of 28
// columns span 28 mask words (29 with the last tile's straddle), so lane l
// ORs word 28 g + l over the tile row's 8 rows and each lane tests its tile
// from two lanes' ORs. A warp takes a run of up to kTileRun groups (of any
// frames; fewer when a launch has too few groups to give every SM a few
// warps, so that a one-frame launch is not a few warps walking long runs):
// each group is a round trip to memory, so the run sets the kernel's length
// (a 64-frame launch: 131 us with runs of 32, 69 with 16, 45 with 8, 49 with
// 4, where the list's one counter starts to take the atomics in turn),
// keeps their ballots, and takes its list space with one atomic: the
// counter is shared by the whole launch, so fewer atomics contend less.
constexpr int kTileRun = 8;

__global__ void __launch_bounds__(256)
lat_tiles(const __grid_constant__ FramePtrs F, int nframes, int env_h, int env_w,
          const uint32_t *__restrict__ final_all, size_t words, uint32_t *__restrict__ list,
          uint32_t *__restrict__ counters, const __grid_constant__ FrameSpans S, int run) {
  const int lane = threadIdx.x & 31;
  // Tile numbers are laid out over the batch's largest frame; each frame has
  // its own tile groups (S) and its own shape bounds its tiles.
  const int ntx = ver_ntx(env_w), nty = ver_nty(env_h);
  const uint32_t ntiles = (uint32_t)ntx * (uint32_t)nty;
  const uint32_t total = (uint32_t)S.start[nframes];
  const uint32_t g0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (uint32_t)run;
  if (g0 >= total)
    return;  // whole warp
  unsigned bal[kTileRun];
  uint32_t first[kTileRun];  // the tile number of each group's first tile
  uint32_t mine = 0, n = 0;
#pragma unroll
  for (int i = 0; i < kTileRun; i++) {
    const uint32_t g = g0 + i;
    bool any = false;
    first[i] = 0;
    if (i < run && g < total) {  // warp-uniform
      const int f = span_frame(S, nframes, (int)g);
      const uint32_t gf = g - (uint32_t)S.start[f];
      const uint32_t ty = fast_div(gf, S.by_row[f]), gx = gf - ty * S.by_row[f].d;
      first[i] = (uint32_t)f * ntiles + ty * (uint32_t)ntx + 32 * gx;
      const uint32_t *fin = final_all + (size_t)f * words;
      const int height = F.h[f], width = F.w[f];
      const int wpr = (width + 31) >> 5;
      const int wd = 28 * (int)gx + lane, r0 = (int)ty * kVerRows;
      uint32_t acc = 0;
      if (lane < 29 && wd < wpr) {
#pragma unroll
        for (int o = 0; o < kVerRows; o++)
          if (r0 + o < height)
            acc |= fin[(size_t)(r0 + o) * wpr + wd];
      }
      const int lw = (kVerTW * lane) >> 5, sh = (kVerTW * lane) & 31;
      const uint32_t lo = __shfl_sync(0xffffffffu, acc, lw);
      const uint32_t hi = __shfl_sync(0xffffffffu, acc, lw + 1);
      const int tx = 32 * (int)gx + lane;
      any = tx < ver_ntx(width) &&
            ((uint32_t)(((unsigned long long)hi << 32 | lo) >> sh) & ((1u << kVerTW) - 1u)) != 0u;
    }
    bal[i] = __ballot_sync(0xffffffffu, any);
    mine |= any ? 1u << i : 0u;
    n += (uint32_t)__popc(bal[i]);
  }
  if (n == 0)
    return;  // whole warp
  uint32_t base = 0;
  if (lane == 0)
    base = atomicAdd(counters + kCtrTiles, n);
  base = __shfl_sync(0xffffffffu, base, 0);
  const unsigned below = (1u << lane) - 1u;
#pragma unroll
  for (int i = 0; i < kTileRun; i++) {
    if ((mine >> i) & 1u)
      list[base + __popc(bal[i] & below)] = first[i] + lane;
    base += (uint32_t)__popc(bal[i]);
  }
}

// Copies listed tile e's pixels and candidate words into buffer s (pieces
// off the frame are written as masked pixels / zero words).
// Copies a tile's pixel rows (r0 - 5 .. r0 + 12, the staged columns from xs)
// into pix (pieces off the frame are written as masked pixels). 16-bit frames
// come here only when 4 | width and they are 8-byte aligned.
template <typename Pix>
__device__ __forceinline__ void stage_pixels(Pix (*pix)[VerPix<Pix>::kPW], const Pix *image,
                                             int height, int width, int vec, int r0, int xs,
                                             int lane) {
  constexpr int kPW = VerPix<Pix>::kPW, kPieces = kPW / 4;
  if (sizeof(Pix) == 2 || vec) {
    // Pieces of 4 pixels, each wholly inside the frame or wholly outside it.
    for (int k = lane; k < kVerPR * kPieces; k += 32) {
      const int r = k / kPieces, ch = k - r * kPieces;
      const int y = r0 - 5 + r, x = xs + 4 * ch;
      Pix *dst = &pix[r][4 * ch];
      if (y >= 0 && y < height && x >= 0 && x + 4 <= width)
        cp_async_piece<Pix>(dst, image + (size_t)y * width + x);
      else
        fill_piece_masked<Pix>(dst);
    }
  } else {
    for (int k = lane; k < kVerPR * kPW; k += 32) {
      const int r = k / kPW, c = k - r * kPW;
      const int y = r0 - 5 + r, x = xs + c;
      Pix *dst = &pix[r][c];
      if (y >= 0 && y < height && x >= 0 && x < width)
        cp_async4(dst, image + (size_t)y * width + x);
      else
        *dst = (Pix)~0u;
    }
  }
}

// The tile's pixels by one TMA box load of frame f's map at (xs, r0 - 5),
// issued by lane 0 once the warp is done with the buffer; it lands on bar.
template <typename Pix>
__device__ __forceinline__ void tma_stage(TileBuf<Pix> &buf, uint64_t *bar, const TileMaps &M,
                                          int f, int r0, int xs, int lane) {
  __syncwarp();
  if (lane == 0) {
    fence_proxy_async_smem();
    mbar_expect_tx(bar, (uint32_t)sizeof(buf.px));
    tma_load_2d(buf.px, &M.map[f], xs, r0 - 5, bar);
  }
}

// Waits for a TMA-staged tile (every lane, bounded; false in every lane if
// any lane's wait ran out) and, for a tile that reaches past the frame, turns
// the box's zero-filled pixels off the frame into masked ones, as the
// per-lane staging writes them.
template <typename Pix>
__device__ __forceinline__ bool tma_landed(TileBuf<Pix> &buf, uint64_t *bar, uint32_t parity,
                                           int height, int width, int r0, int xs, int lane) {
  constexpr int kPW = VerPix<Pix>::kPW;
  if (!__all_sync(0xffffffffu, mbar_wait(bar, parity)))
    return false;
  const int y0 = r0 - 5;
  if (y0 < 0 || y0 + kVerPR > height || xs < 0 || xs + kPW > width) {  // warp-uniform
    for (int k = lane; k < kVerPR * kPW; k += 32) {
      const int r = k / kPW, c = k - r * kPW;
      const int y = y0 + r, x = xs + c;
      if (y < 0 || y >= height || x < 0 || x >= width)
        buf.px[r][c] = (Pix)~0u;
    }
  }
  __syncwarp();
  return true;
}

// The tile origin of list entry e: frame, first output row and column.
struct TileAt {
  int f, r0, c0;
};
__device__ __forceinline__ TileAt tile_at(uint32_t e, uint32_t ntiles, int ntx,
                                          const FastDiv &by_ntiles, const FastDiv &by_ntx) {
  const uint32_t fu = fast_div(e, by_ntiles), t = e - fu * ntiles, tyu = fast_div(t, by_ntx);
  TileAt a;
  a.f = (int)fu;
  a.r0 = (int)tyu * kVerRows;
  a.c0 = (int)(t - tyu * (uint32_t)ntx) * kVerTW;
  return a;
}
// The staged columns' first column (aligned) for a tile starting at c0.
template <typename Pix> __device__ __forceinline__ int tile_xs(int c0) {
  return (c0 - 5) & ~(VerPix<Pix>::kAlign - 1);
}

template <typename Pix>
__device__ __forceinline__ void ver_stage(VerWarp<Pix> &sm, int s, uint32_t e, const FramePtrs &F,
                                          const TileMaps &M, int tma, int vec, uint32_t ntiles,
                                          int ntx, const FastDiv &by_ntiles,
                                          const FastDiv &by_ntx,
                                          const uint32_t *__restrict__ final_all,
                                          size_t words, int lane) {
  const TileAt a = tile_at(e, ntiles, ntx, by_ntiles, by_ntx);
  const int f = a.f, r0 = a.r0, c0 = a.c0;
  const int height = F.h[f], width = F.w[f];
  const int xs = tile_xs<Pix>(c0);
  __syncwarp();  // every lane is done with the pixel buffer
  if (tma)
    tma_stage<Pix>(sm.pix[0], &sm.bar[0], M, f, r0, xs, lane);
  else
    stage_pixels<Pix>(sm.pix[0].px, reinterpret_cast<const Pix *>(F.image[f]), height, width,
                      vec, r0, xs, lane);
  if (lane < 2 * kVerRows) {
    const int o = lane >> 1, wdx = (c0 >> 5) + (lane & 1);
    const int wpr = (width + 31) >> 5;
    uint32_t *dst = &sm.cw[s][o][lane & 1];
    if (r0 + o < height && wdx < wpr)
      cp_async4(dst, final_all + (size_t)f * words + (size_t)(r0 + o) * wpr + wdx);
    else
      *dst = 0u;
  }
}

// The packed sums of the stage-0 window of row d, column `col` of a tile
// (seven column sums of seven rows; a window holds 49 pixels, so its masked
// count m <= 49 -- callers clamp it anyway, which keeps the per-count tables
// in bounds whatever the sums).
template <typename Pix>
__device__ __forceinline__ void ver_window(const VerWarp<Pix> &sm, int d, int col, uint32_t *Wn,
                                           uint32_t *Wq) {
  uint32_t n = 0, q = 0;
#pragma unroll
  for (int u = 0; u <= 2 * kLatK; u++) {
    const uint2 x = sm.vs[d][col + u];
    n += x.x;
    q += x.y;
  }
  *Wn = n;
  *Wq = q;
}

template <int kOcc, typename Pix>
__global__ void __launch_bounds__(kVerWarps * 32, kOcc)
lat_verify(const __grid_constant__ FramePtrs F, const __grid_constant__ TileMaps M, int tma,
           int env_h, int env_w, int vec, const __grid_constant__ LaunchParams P,
           const __grid_constant__ StreamTables T, uint32_t *__restrict__ final_all, size_t words,
           const uint32_t *__restrict__ list,
           uint32_t *__restrict__ counters, FastDiv by_ntiles, FastDiv by_ntx,
           uint32_t *__restrict__ list2) {
  extern __shared__ __align__(128) unsigned char ver_smem_raw[];
  // The launch gives 128 bytes more than the layout needs: the tile buffers
  // start on a 128-byte boundary whatever the base's alignment.
  unsigned char *ver_smem = ver_smem_raw + ((128u - (smem_addr(ver_smem_raw) & 127u)) & 127u);
  uint4 *tab = reinterpret_cast<uint4 *>(ver_smem);
  constexpr bool k16 = sizeof(Pix) == 2;
  VerWarp<Pix> *warps = reinterpret_cast<VerWarp<Pix> *>(ver_smem + sizeof(uint4) * 64);
  for (int m = threadIdx.x; m <= kLatN0; m += blockDim.x)
    tab[m] = make_uint4(T.nk[kLatN0 - m], T.clo[kLatN0 - m], T.chi[kLatN0 - m], 0u);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  VerWarp<Pix> &sm = warps[warp];
  if (tma && lane == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init_fence();
  }
  __syncthreads();
  uint32_t parity = 0;  // bit b: the phase the next wait on bar[b] waits for
  // Tile numbers are laid out over the batch's largest frame.
  const int ntx = ver_ntx(env_w);
  const uint32_t ntiles = (uint32_t)ntx * (uint32_t)ver_nty(env_h);
  const uint32_t narrow2 = T.narrow_max + 2u;
  const uint32_t count = counters[kCtrTiles];
  const uint32_t nw = gridDim.x * kVerWarps;
  uint32_t k = blockIdx.x * kVerWarps + warp;
  // List entries are read a tile before they are staged. A warp has one
  // pixel buffer: the next tile's load goes out as soon as this tile's pixels
  // have been read (after the column sums, or after the windows summed from
  // the pixels on a frame with very large counts), and runs under the rest of
  // this tile's check. The candidate words are staged into the other of two.
  uint32_t e = k < count ? list[k] : 0u;
  uint32_t e1 = k + nw < count ? list[k + nw] : 0u;
  if (k < count)
    ver_stage<Pix>(sm, 0, e, F, M, tma, vec, ntiles, ntx, by_ntiles, by_ntx, final_all, words,
                   lane);
  cp_async_commit();
  uint32_t e2 = 0u;
  uint32_t inflight = k < count ? 1u : 0u;  // a TMA load not waited for
  for (int s = 0; k < count; k += nw, s ^= 1, e = e1, e1 = e2) {
    e2 = k + 2 * nw < count ? list[k + 2 * nw] : 0u;
    cp_async_wait<0>();  // this tile's pieces have landed
    __syncwarp();
    const TileAt a = tile_at(e, ntiles, ntx, by_ntiles, by_ntx);
    const int f = a.f, r0 = a.r0, c0 = a.c0;
    const int height = F.h[f], width = F.w[f], wpr = (width + 31) >> 5;
    if (tma) {
      inflight = 0u;
      if (!tma_landed<Pix>(sm.pix[0], &sm.bar[0], parity & 1u, height, width, r0,
                           tile_xs<Pix>(c0), lane)) {
        if (lane == 0)
          atomicOr(counters + kCtrFault, 1u);
        break;  // whole warp
      }
      parity ^= 1u;
    }
    // The next tile's load, once this tile's pixels have been read.
    auto stage_next = [&]() {
      if (k + nw < count) {
        ver_stage<Pix>(sm, s ^ 1, e1, F, M, tma, vec, ntiles, ntx, by_ntiles, by_ntx,
                       final_all, words, lane);
        inflight = 1u;
      }
      cp_async_commit();
    };
    const int off = (c0 - 5) - tile_xs<Pix>(c0);
    const int w0 = c0 >> 5, sh = c0 & 31;
    uint32_t cj[kVerRows];
#pragma unroll
    for (int o = 0; o < kVerRows; o++) {
      const unsigned long long x =
          (unsigned long long)sm.cw[s][o][0] | (unsigned long long)sm.cw[s][o][1] << 32;
      cj[o] = (uint32_t)(x >> sh) & ((1u << kVerTW) - 1u);
    }
    // Columns B (pixel columns 32-37, stage-0 columns 26-31) matter only
    // when a candidate lies in the tile's last 6 columns.
    uint32_t late = 0;
#pragma unroll
    for (int o = 0; o < kVerRows; o++)
      late |= cj[o] >> 22;
    const int npass = late ? 2 : 1;
    // Pixel columns off + lane (A) and off + 32 + lane (B, lanes 0-5): the
    // masked pixels by row, the largest valid one, and the column sums of 7
    // rows for the 12 stage-0 rows (exact in 32 bits unless the tile holds a
    // valid pixel at or above narrow_max, which the check below catches).
    uint32_t mx = 0;
#pragma unroll
    for (int pass = 0; pass < 2; pass++) {
      if (pass == npass)
        break;  // warp-uniform
      if (pass == 1 && lane >= kVerPC - 32)
        break;
      const int col = off + 32 * pass + lane;
      uint32_t ns[kVerPR], q[kVerPR], mk = 0;
#pragma unroll
      for (int r = 0; r < kVerPR; r++) {
        const uint32_t v = sm.pix[0].px[r][col];
        const bool masked = is_masked_px<Pix>(v);
        if (!k16)
          mx = max(mx, v + 2u);
        mk |= (masked ? 1u : 0u) << r;
        ns[r] = masked ? (1u << kLatPS) : v;
        q[r] = ns[r] * ns[r];
      }
      sm.msk[32 * pass + lane] = mk;
      uint32_t cn = 0, cq = 0;
#pragma unroll
      for (int r = 0; r < 2 * kLatK; r++) {
        cn += ns[r];
        cq += q[r];
      }
#pragma unroll
      for (int d = 0; d < kVerDR; d++) {
        cn += ns[d + 2 * kLatK];
        cq += q[d + 2 * kLatK];
        sm.vs[d][32 * pass + lane] = make_uint2(cn, cq);
        cn -= ns[d];
        cq -= q[d];
      }
    }
    __syncwarp();
    // 16-bit frames sum in 32 bits as the reference does: never wide.
    const bool wide = !k16 && __any_sync(0xffffffffu, mx >= narrow2);
    if (!wide)
      stage_next();  // the windows come from the column sums, not the pixels
    if (wide && lane == 0)
      counters[kCtrBatch + (size_t)f * kCtrCount + kCtrWideFrame] = 1u;
    // The stage-0 positions within 2 of a candidate: lane d first forms row
    // d's (row r0 - 2 + d, bit = column c0 - 2 + bit), then every lane takes
    // its own column's rows of them, less those whose centre is masked (set
    // whatever the window).
    uint32_t need = 0;
#pragma unroll
    for (int o = 0; o < kVerRows; o++)
      need |= (o >= lane - 4 && o <= lane) ? cj[o] : 0u;
    {
      const uint32_t x2 = need | need << 1;
      need = lane < kVerDR ? (x2 | x2 << 2 | need << 4) : 0u;
    }
    uint32_t rows = 0;
#pragma unroll
    for (int d = 0; d < kVerDR; d++)
      rows |= ((__shfl_sync(0xffffffffu, need, d) >> lane) & 1u) << d;
    rows &= ~(sm.msk[lane + kLatK] >> kLatK);
    // Each lane decides its column's needed windows (lane = column, so no
    // two lanes share a result bit): a row's bit clears when its window is
    // not signal.
    uint32_t keep = 0xFFFFFFFFu;  // bit d: row d's window here is signal (or not needed)
    if constexpr (k16) {
      // The reference's float test of every needed window, exactly.
      while (rows) {
        const int d = __ffs(rows) - 1;
        rows &= rows - 1u;
        uint32_t Wn, Wq;
        ver_window(sm, d, lane, &Wn, &Wq);
        const uint32_t m = min(Wn >> kLatPS, (uint32_t)kLatN0);
        if (!stage0_u16((uint32_t)kLatN0 - m, Wn & kLatMask, Wq, P))
          keep &= ~(1u << d);
      }
    } else if (wide) {
      // 64-bit sums from the staged tile (frames with very large counts).
      while (rows) {
        const int d = __ffs(rows) - 1;
        rows &= rows - 1u;
        if (!lat_wide(reinterpret_cast<const uint32_t (*)[kVerPW]>(sm.pix[0].px), d,
                      off + lane, P))
          keep &= ~(1u << d);
      }
    } else {
      // The two bounds first; the windows between them (rare) are decided by
      // the reference's sequence afterwards, out of the loop.
      uint32_t amb = 0;
      while (rows) {
        const int d = __ffs(rows) - 1;
        rows &= rows - 1u;
        uint32_t Wn, Wq;
        ver_window(sm, d, lane, &Wn, &Wq);
        const uint32_t m = min(Wn >> kLatPS, (uint32_t)kLatN0), S = Wn & kLatMask;
        const uint4 c = tab[m];
        const unsigned long long L = (unsigned long long)Wq * c.x;
        const bool maybe = L > (unsigned long long)S * ((S << kDec) + c.y);
        const bool sure = L >= (unsigned long long)S * ((S << kDec) + c.z) + (2ull << kDec);
        keep &= maybe ? ~0u : ~(1u << d);
        amb |= (maybe && !sure) ? 1u << d : 0u;
      }
      while (amb) {
        const int d = __ffs(amb) - 1;
        amb &= amb - 1u;
        uint32_t Wn, Wq;
        ver_window(sm, d, lane, &Wn, &Wq);
        const uint32_t m = min(Wn >> kLatPS, (uint32_t)kLatN0);
        if (!lat_exact((uint32_t)kLatN0 - m, Wn & kLatMask, Wq, P))
          keep &= ~(1u << d);
      }
    }
    if (wide)
      stage_next();
    uint32_t D[kVerDR];
#pragma unroll
    for (int d = 0; d < kVerDR; d++)
      D[d] = __ballot_sync(0xffffffffu, (keep >> d) & 1u);
    __syncwarp();  // the next tile rewrites the shared rows
    // The exact erosion of the tile's rows; the candidates that fail leave
    // the mask, and a tile with a candidate left goes on stage 2's list.
    uint32_t *fin = final_all + (size_t)f * words;
    uint32_t left = 0;
#pragma unroll
    for (int o = 0; o < kVerRows; o++) {
      uint32_t V = 0xFFFFFFFFu;
#pragma unroll
      for (int u = 0; u < 5; u++)
        V &= D[o + u];
      uint32_t H = V;
#pragma unroll
      for (int u = 1; u < 5; u++)
        H &= V >> u;
      left |= cj[o] & H;
      const uint32_t clear = cj[o] & ~H;
      if (clear && lane < 2) {
        const unsigned long long c64 = (unsigned long long)clear << sh;
        const uint32_t part = (uint32_t)(c64 >> (32 * lane));
        if (part && w0 + lane < wpr) {
          const size_t at = (size_t)(r0 + o) * wpr + w0 + lane;
          atomicAnd(fin + at, ~part);
        }
      }
    }
    if (lane == 0)
      list2[k] = left ? e : kNoTile;  // same place as in the tile list: no atomics
  }
  // After a fault: the load still in flight (bounded) before the buffer goes.
  if (tma && inflight)
    (void)mbar_wait(&sm.bar[0], parity & 1u);
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// Stage 2 (src/spots/dext.cc:151-222) on the listed tiles, after the exact
// check: a candidate's background is the valid pixels of its clipped 11 x 11
// window outside the eroded mask, and the tile's 18 x 38 pixels hold every
// window of its candidates. A warp stages them with the candidate-mask words
// over them (cp.async, the next tile's while it works on this one; a pixel is
// in the eroded mask when its bit is set or it is masked), takes
// column sums of 11 rows once per tile, then per candidate adds 11 of them
// and runs the reference's test (sf_common.cuh). The result goes to the
// candidate's place in the ascending candidate list, from the per-word list
// positions of the candidate mask (mask_prefix); the mask itself is left as
// it is until every position is taken (pass_sums clears the failures).
// ---------------------------------------------------------------------------
template <typename Pix> struct alignas(128) S2Warp {
  TileBuf<Pix> pix[2];              // staged pixels, two tiles
  uint64_t bar[2];                  // their TMA mbarriers
  uint32_t ew[2][kVerPR][3];        // candidate-mask words over the staged columns
  uint32_t cw[2][kVerRows][2];      // candidate-mask words of the tile's rows
  uint32_t pw[2][kVerRows][2];      // their list positions
  uint2 cs[kVerRows][kVerPC + 2];   // {count, sum} of 11 rows of background
};

template <typename Pix>
__device__ __forceinline__ void s2_stage(S2Warp<Pix> &sm, int s, uint32_t e, const FramePtrs &F,
                                         const TileMaps &M, int tma, int vec, uint32_t ntiles,
                                         int ntx, const FastDiv &by_ntiles,
                                         const FastDiv &by_ntx,
                                         const uint32_t *__restrict__ final_all,
                                         const uint32_t *__restrict__ prefix_all, size_t words,
                                         int lane) {
  const TileAt a = tile_at(e, ntiles, ntx, by_ntiles, by_ntx);
  const int f = a.f, r0 = a.r0, c0 = a.c0;
  const int height = F.h[f], width = F.w[f];
  const int xs = tile_xs<Pix>(c0);
  if (tma)
    tma_stage<Pix>(sm.pix[s], &sm.bar[s], M, f, r0, xs, lane);
  else
    stage_pixels<Pix>(sm.pix[s].px, reinterpret_cast<const Pix *>(F.image[f]), height, width,
                      vec, r0, xs, lane);
  const int wpr = (width + 31) >> 5;
  const uint32_t *fin = final_all + (size_t)f * words;
  for (int k = lane; k < kVerPR * 3; k += 32) {
    const int r = k / 3, j = k - 3 * r;
    const int y = r0 - 5 + r, wd = (xs >> 5) + j;
    uint32_t *dst = &sm.ew[s][r][j];
    if (y >= 0 && y < height && wd >= 0 && wd < wpr)
      cp_async4(dst, fin + (size_t)y * wpr + wd);
    else
      *dst = 0u;
  }
  if (lane < 2 * kVerRows) {
    const int o = lane >> 1, wdx = (c0 >> 5) + (lane & 1);
    const bool in = r0 + o < height && wdx < wpr;
    const size_t at = (size_t)f * words + (size_t)(r0 + o) * wpr + wdx;
    if (in) {
      cp_async4(&sm.cw[s][o][lane & 1], final_all + at);
      cp_async4(&sm.pw[s][o][lane & 1], prefix_all + at);
    } else {
      sm.cw[s][o][lane & 1] = 0u;
      sm.pw[s][o][lane & 1] = 0u;
    }
  }
}

template <int kOcc, typename Pix>
__global__ void __launch_bounds__(kVerWarps * 32, kOcc)
lat_stage2(const __grid_constant__ FramePtrs F, const __grid_constant__ TileMaps M, int tma,
           int env_h, int env_w, int vec, const __grid_constant__ LaunchParams P,
           const uint32_t *__restrict__ final_all, const uint32_t *__restrict__ prefix_all,
           size_t words,
           const uint32_t *__restrict__ list, uint32_t *__restrict__ counters,
           uint32_t *__restrict__ cand_all, uint2 *__restrict__ res_all, uint32_t cand_cap,
           FastDiv by_ntiles, FastDiv by_ntx) {
  extern __shared__ __align__(128) unsigned char s2_smem_raw[];
  // 128 bytes more than the layout: the tile buffers start on a 128-byte
  // boundary whatever the base's alignment.
  unsigned char *s2_smem = s2_smem_raw + ((128u - (smem_addr(s2_smem_raw) & 127u)) & 127u);
  constexpr bool k16 = sizeof(Pix) == 2;
  // A fault in the exact check leaves its tile list partly unwritten: nothing
  // to do (the launch's counts report the fault).
  if (counters[kCtrFault])
    return;
  S2Warp<Pix> &sm = reinterpret_cast<S2Warp<Pix> *>(s2_smem)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  if (tma && lane == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    mbar_init_fence();
  }
  __syncwarp();
  uint32_t parity = 0;  // bit b: the phase the next wait on bar[b] waits for
  // Tile numbers are laid out over the batch's largest frame.
  const int ntx = ver_ntx(env_w);
  const uint32_t ntiles = (uint32_t)ntx * (uint32_t)ver_nty(env_h);
  // The exact check's tile list with the tiles left without a candidate
  // marked kNoTile; a warp takes every nw-th entry and stages the next one it
  // will check while it checks the current one.
  const uint32_t count = counters[kCtrTiles];
  const uint32_t nw = gridDim.x * kVerWarps;
  auto next_live = [&](uint32_t from, uint32_t *at) {
    uint32_t x = kNoTile;
    for (; from < count; from += nw) {
      x = list[from];
      if (x != kNoTile)
        break;
    }
    *at = from;
    return from < count ? x : kNoTile;
  };
  uint32_t k, k1;
  uint32_t e = next_live(blockIdx.x * kVerWarps + (threadIdx.x >> 5), &k);
  uint32_t e1 = next_live(k + nw, &k1);
  if (k < count)
    s2_stage<Pix>(sm, 0, e, F, M, tma, vec, ntiles, ntx, by_ntiles, by_ntx, final_all,
                  prefix_all, words, lane);
  cp_async_commit();
  uint32_t inflight = k < count ? 1u : 0u;  // bit b: a TMA load into buffer b not waited for
  for (int s = 0; k < count; s ^= 1) {
    if (k1 < count) {
      s2_stage<Pix>(sm, s ^ 1, e1, F, M, tma, vec, ntiles, ntx, by_ntiles, by_ntx, final_all,
                    prefix_all, words, lane);
      inflight |= 2u >> s;
    }
    cp_async_commit();
    cp_async_wait<1>();
    __syncwarp();
    const TileAt a = tile_at(e, ntiles, ntx, by_ntiles, by_ntx);
    const int f = a.f, r0 = a.r0, c0 = a.c0;
    const int height = F.h[f], width = F.w[f];
    const int xs = tile_xs<Pix>(c0), off = (c0 - 5) - xs;
    if (tma) {
      inflight &= ~(1u << s);
      if (!tma_landed<Pix>(sm.pix[s], &sm.bar[s], (parity >> s) & 1u, height, width, r0, xs,
                           lane)) {
        if (lane == 0)
          atomicOr(counters + kCtrFault, 1u);
        break;  // whole warp
      }
      parity ^= 1u << s;
    }
    const int w0 = c0 >> 5, sh = c0 & 31;
    uint32_t cj[kVerRows], late = 0;
    int incl = 0;
#pragma unroll
    for (int o = 0; o < kVerRows; o++) {
      const unsigned long long x =
          (unsigned long long)sm.cw[s][o][0] | (unsigned long long)sm.cw[s][o][1] << 32;
      cj[o] = (uint32_t)(x >> sh) & ((1u << kVerTW) - 1u);
      late |= cj[o] >> 22;
      incl += __popc(cj[o]);
    }
    const int total = incl;  // the tile's candidates (the same in every lane)
    if (total == 0) {
      __syncwarp();
      k = k1;
      e = e1;
      e1 = next_live(k1 + nw, &k1);
      continue;
    }
    // Background by column: A = staged column off + lane, B = off + 32 + lane
    // (needed only for candidates in the tile's last 6 columns). Valid
    // pixels below 2^24 keep the sums of 121 of them within 32 bits; a tile
    // holding a larger one sums each window in 64 bits instead.
    uint32_t mx = 0;
    const int npass = late ? 2 : 1;
#pragma unroll
    for (int pass = 0; pass < 2; pass++) {
      if (pass == npass)
        break;
      if (pass == 1 && lane >= kVerPC - 32)
        break;
      const int j = off + 32 * pass + lane;
      const int x = xs + j, wi = (x >> 5) - (xs >> 5), b = x & 31;
      uint32_t bn[kVerPR], bs[kVerPR];
#pragma unroll
      for (int r = 0; r < kVerPR; r++) {
        const uint32_t v = sm.pix[s].px[r][j];
        const bool eroded = (sm.ew[s][r][wi] >> b) & 1u;
        const bool bg = !is_masked_px<Pix>(v) && !eroded;
        if (!k16)
          mx = max(mx, v + 2u);
        bn[r] = bg ? 1u : 0u;
        bs[r] = bg ? v : 0u;
      }
      uint32_t cn = 0, cs = 0;
#pragma unroll
      for (int r = 0; r < 10; r++) {
        cn += bn[r];
        cs += bs[r];
      }
#pragma unroll
      for (int o = 0; o < kVerRows; o++) {
        cn += bn[o + 10];
        cs += bs[o + 10];
        sm.cs[o][32 * pass + lane] = make_uint2(cn, cs);
        cn -= bn[o];
        cs -= bs[o];
      }
    }
    // 121 16-bit pixels sum below 2^23: 16-bit frames are never wide.
    const bool wide = !k16 && __any_sync(0xffffffffu, mx >= (1u << 24) + 2u);
    __syncwarp();
    // The tile's candidates, spread over the lanes in order.
    int pre[kVerRows];
    {
      int run = 0;
#pragma unroll
      for (int o = 0; o < kVerRows; o++) {
        pre[o] = run;
        run += __popc(cj[o]);
      }
    }
    uint32_t *cand = cand_all + (size_t)f * cand_cap;
    uint2 *res = res_all + (size_t)f * cand_cap;
    for (int q = lane; q < total; q += 32) {
      int o = 0;
#pragma unroll
      for (int e2 = 1; e2 < kVerRows; e2++)
        o += q >= pre[e2] ? 1 : 0;
      uint32_t bits = 0;
#pragma unroll
      for (int e2 = 0; e2 < kVerRows; e2++)
        bits = e2 == o ? cj[e2] : bits;
      const int tcol = (int)__fns(bits, 0u, q - pre[o] + 1);
      uint32_t n = 0;
      unsigned long long S = 0;
      if (!wide) {
        uint32_t s32 = 0;
#pragma unroll
        for (int u = 0; u < 11; u++) {
          const uint2 c = sm.cs[o][tcol + u];
          n += c.x;
          s32 += c.y;
        }
        S = s32;
      } else {
        for (int r = o; r < o + 11; r++)
          for (int u = 0; u < 11; u++) {
            const int j = off + tcol + u, x = xs + j;
            const uint32_t v = sm.pix[s].px[r][j];
            const bool eroded = (sm.ew[s][r][(x >> 5) - (xs >> 5)] >> (x & 31)) & 1u;
            if (!is_masked_px<Pix>(v) && !eroded) {
              n++;
              S += v;
            }
          }
      }
      const uint32_t p = sm.pix[s].px[o + 5][off + tcol + 5];
      float bg = 0.0f;
      // dext.cc:205: only pixels above the global threshold are tested.
      bool sig = (uint64_t)p >= P.p_min;
      if (sig) {
        if constexpr (k16)
          sig = stage2_u16(p, n, (uint32_t)S, P, &bg);  // the reference's float test
        else
          sig = stage2_u32(p, n, S, P, &bg);
      }
      const int x = c0 + tcol, jw = (x >> 5) - w0, bit = x & 31;
      const uint32_t i = sm.pw[s][o][jw] + (uint32_t)__popc(sm.cw[s][o][jw] & ((1u << bit) - 1u));
      if (i < cand_cap) {
        cand[i] = (uint32_t)(r0 + o) * (uint32_t)width + (uint32_t)x;
        res[i] = make_uint2(__float_as_uint(bg), n | (sig ? 1u << 16 : 0u));
      }
    }
    __syncwarp();  // the next tile rewrites the shared sums
    k = k1;
    e = e1;
    e1 = next_live(k1 + nw, &k1);
  }
  // After a fault: the load still in flight (bounded) before the buffers go.
  for (int b = 0; b < 2; b++)
    if (tma && ((inflight >> b) & 1u))
      (void)mbar_wait(&sm.bar[b], (parity >> b) & 1u);
  cp_async_wait<0>();
}

// Both add 128 bytes for aligning the tile buffers (see the kernels).
template <typename Pix> constexpr size_t s2_smem_bytes() {
  return sizeof(S2Warp<Pix>) * kVerWarps + 128;
}

template <typename Pix> constexpr size_t ver_smem_bytes() {
  return sizeof(uint4) * 64 + sizeof(VerWarp<Pix>) * kVerWarps + 128;
}
static_assert(sizeof(uint4) * 64 % 128 == 0, "the verify warps start 128-byte aligned");
static_assert((ver_smem_bytes<uint32_t>() + 1024) * kVerOcc <= 228 * 1024,
              "six exact-check blocks an SM");

int lat_slots() {
  static int slots = 0;
  if (!slots) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lat_stage01<kLatOcc, true, uint32_t>,
                                                  kLatWarps * 32, ring_bytes<uint32_t>());
    slots = std::max(1, per) * kLatWarps * device_sms();
  }
  return slots;
}

// Blocks an SM of a persistent kernel with `bytes` of dynamic shared memory,
// once per instantiation (the attribute set first).
template <class Kernel> cudaError_t persistent_blocks(Kernel k, size_t bytes, int *blocks) {
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  int per = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, kVerWarps * 32, bytes);
  *blocks = std::max(1, per);
  return e;
}

// The launch's frames mapped for the TMA staging of tiles (1), or not
// mappable (0: a frame not 16-byte aligned, a row pitch that is not a
// multiple of 16 bytes, no driver entry point), the per-lane staging then.
template <typename Pix> int make_tile_maps(const FramePtrs &F, int nframes, int h, int w,
                                           TileMaps *M) {
  std::memset(M, 0, sizeof(*M));
  for (int f = 0; f < nframes; f++)
    if (!encode_frame_map(&M->map[f], F.image[f], F.h[f], F.w[f], (int)sizeof(Pix),
                          VerPix<Pix>::kPW, kVerPR))
      return 0;
  return 1;
}

template <typename Pix>
cudaError_t lattice_stage2(const FramePtrs &F, int nframes, int h, int w, int vec,
                           const LaunchParams &P, const StreamBuffers &b, cudaStream_t stream) {
  static std::once_flag configured;
  static cudaError_t config_error = cudaSuccess;
  static int blocks = 0;
  std::call_once(configured, [] {
    config_error = persistent_blocks(lat_stage2<kS2Occ, Pix>, s2_smem_bytes<Pix>(), &blocks);
  });
  if (config_error != cudaSuccess)
    return config_error;
  // The tiles the exact check left a candidate in (its second list).
  const uint32_t *prefix = b.amb;
  const size_t tiles = (size_t)ver_ntx(w) * (size_t)ver_nty(h);
  const uint32_t *list = b.amb + (size_t)nframes * (b.words + tiles);
  TileMaps M;
  const int tma = make_tile_maps<Pix>(F, nframes, h, w, &M);
  lat_stage2<kS2Occ, Pix><<<blocks * device_sms(), kVerWarps * 32, s2_smem_bytes<Pix>(),
                             stream>>>(F, M, tma, h, w, vec, P, b.bits, prefix, b.words,
                                       list, b.counters, b.cand, b.res, b.cand_cap,
                                       make_fastdiv((uint32_t)tiles),
                                       make_fastdiv((uint32_t)ver_ntx(w)));
  return cudaGetLastError();
}

// Strips of a frame w wide (whole mask rows: the last strip reaches the end
// of the row's last word).
int lat_strips(int w) { return ((w + 31) / 32 * 32 + kLatOut - 1) / kLatOut; }

template <typename Pix>
cudaError_t lattice(const FramePtrs &F, int nframes, int h, int w, int vec, const LaunchParams &P,
                    const StreamTables &T, const StreamBuffers &b, int run_rows,
                    cudaStream_t stream) {
  // Each frame's strips x runs of run_rows rows, frame after frame.
  FrameSpans S;
  S.start[0] = 0;
  for (int f = 0; f < nframes; f++) {
    const int strips = lat_strips(F.w[f]);
    S.start[f + 1] = S.start[f] + strips * ((F.h[f] + run_rows - 1) / run_rows);
    S.by_row[f] = make_fastdiv((uint32_t)strips);
  }
  const size_t mask_bytes = b.words * sizeof(uint32_t);
  const unsigned lb = (unsigned)((S.start[nframes] + kLatWarps - 1) / kLatWarps);
  uint8_t *fin = reinterpret_cast<uint8_t *>(b.bits);
  if (sizeof(Pix) == 2 || vec)
    lat_stage01<kLatOcc, true, Pix><<<lb, kLatWarps * 32, ring_bytes<Pix>(), stream>>>(
        F, nframes, vec, S, run_rows, T, P, fin, mask_bytes);
  else
    lat_stage01<kLatOcc, false, uint32_t><<<lb, kLatWarps * 32, 0, stream>>>(
        F, nframes, vec, S, run_rows, T, P, fin, mask_bytes);
  static std::once_flag configured;
  static cudaError_t config_error = cudaSuccess;
  static int ver_blocks = 0;
  std::call_once(configured, [] {
    config_error = persistent_blocks(lat_verify<kVerOcc, Pix>, ver_smem_bytes<Pix>(),
                                     &ver_blocks);
  });
  if (config_error != cudaSuccess)
    return config_error;
  // The ambiguous-mask buffer of the other streaming path holds, here, the
  // candidate mask's per-word list positions (stage 2), the tile list and the
  // list of tiles the exact check leaves a candidate in.
  // Tile groups: each frame's tile rows x groups of 32 tiles.
  FrameSpans G;
  G.start[0] = 0;
  for (int f = 0; f < nframes; f++) {
    const int ngx = (ver_ntx(F.w[f]) + 31) / 32;
    G.start[f + 1] = G.start[f] + ver_nty(F.h[f]) * ngx;
    G.by_row[f] = make_fastdiv((uint32_t)ngx);
  }
  const long long tgroups = G.start[nframes];
  // Runs of kTileRun groups a warp, shorter when that would leave fewer than
  // 8 warps an SM (one frame: runs of 2).
  const int trun = (int)std::max(1ll, std::min((long long)kTileRun,
                                               tgroups / (8ll * device_sms())));
  const long long twarps = (tgroups + trun - 1) / trun;
  const unsigned tb = (unsigned)((twarps + 7) / 8);
  const size_t tiles = (size_t)ver_ntx(w) * (size_t)ver_nty(h);
  uint32_t *list = b.amb + (size_t)nframes * b.words;
  const FastDiv by_ntiles = make_fastdiv((uint32_t)tiles);
  const FastDiv by_ntx = make_fastdiv((uint32_t)ver_ntx(w));
  lat_tiles<<<tb, 256, 0, stream>>>(F, nframes, h, w, b.bits, b.words, list, b.counters, G,
                                    trun);
  TileMaps M;
  const int tma = make_tile_maps<Pix>(F, nframes, h, w, &M);
  lat_verify<kVerOcc, Pix><<<ver_blocks * device_sms(), kVerWarps * 32, ver_smem_bytes<Pix>(),
                             stream>>>(F, M, tma, h, w, vec, P, T, b.bits, b.words, list,
                                       b.counters, by_ntiles, by_ntx,
                                       list + (size_t)nframes * tiles);
  return cudaGetLastError();
}

} // namespace

bool encode_frame_map(CUtensorMap *map, const void *base, int h, int w, int bytes_per_pixel,
                      int box_w, int box_h) {
  // The driver's encoder, looked up once (no link against libcuda).
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      fn = nullptr;
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  const size_t pitch = (size_t)w * (size_t)bytes_per_pixel;
  if (!encode || !base || reinterpret_cast<uintptr_t>(base) % 16 != 0 || pitch % 16 != 0 ||
      h < 1 || w < 1 || (bytes_per_pixel != 2 && bytes_per_pixel != 4))
    return false;
  const cuuint64_t dims[2] = {(cuuint64_t)w, (cuuint64_t)h};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch};
  const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
  const cuuint32_t step[2] = {1, 1};
  return encode(map,
                bytes_per_pixel == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32
                                     : CU_TENSOR_MAP_DATA_TYPE_UINT16,
                2, const_cast<void *>(base), dims, strides, box, step,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t lattice_tiles(int h, int w) { return (size_t)ver_ntx(w) * (size_t)ver_nty(h); }

cudaError_t launch_lattice_stage2(const FramePtrs &F, int nframes, int h, int w, int vec,
                                  int pixel_bytes, const LaunchParams &P, const StreamBuffers &b,
                                  cudaStream_t stream) {
  return pixel_bytes == 2 ? lattice_stage2<uint16_t>(F, nframes, h, w, vec, P, b, stream)
                          : lattice_stage2<uint32_t>(F, nframes, h, w, vec, P, b, stream);
}

// The run length for a launch whose tallest frame has h rows and whose
// frames have `strips` strips in all: the resident warps filled once (no
// tail wave) by the tallest frame's runs, unless run_rows is given; at least
// kMinRunRows, in whole triples of rows.
static int lat_run_rows(int h, long long strips, int run_rows) {
  if (run_rows <= 0) {
    const long long nruns = std::max(1ll, (long long)lat_slots() / std::max(1ll, strips));
    run_rows = (int)((h + nruns - 1) / nruns);
  }
  run_rows = std::max(run_rows, kMinRunRows);
  return (run_rows + 2) / 3 * 3;
}

LatticeGeometry lattice_geometry(int h, int w, int nframes, int run_rows) {
  LatticeGeometry g;
  g.nstrips = lat_strips(w);
  g.run_rows = lat_run_rows(h, (long long)nframes * g.nstrips, run_rows);
  g.nruns = (h + g.run_rows - 1) / g.run_rows;
  return g;
}

cudaError_t launch_lattice(const FramePtrs &F, int nframes, int h, int w, int vec,
                           int pixel_bytes, const LaunchParams &P, const StreamTables &T,
                           const StreamBuffers &b, int run_rows, cudaStream_t stream) {
  if (P.half != kLatK)
    return cudaErrorInvalidValue;
  long long strips = 0;
  for (int f = 0; f < nframes; f++)
    strips += lat_strips(F.w[f]);
  const int rr = lat_run_rows(h, strips, run_rows);
  return pixel_bytes == 2 ? lattice<uint16_t>(F, nframes, h, w, vec, P, T, b, rr, stream)
                          : lattice<uint32_t>(F, nframes, h, w, vec, P, T, b, rr, stream);
}

} // namespace sf
