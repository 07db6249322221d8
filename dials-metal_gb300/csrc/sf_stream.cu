// The streaming threshold for 32-bit frames (the benchmark path), for one
// frame or a batch of same-shaped frames per launch sequence.
//
// Stage 0 and the erosion of src/spots/dext.cc (:53-142) run in one pass in
// which every warp walks down its own strip of rows; stage 2 (:151-222) runs
// afterwards only at the candidates the erosion leaves, a percent or so of
// the frame:
//
//   seg_stage01   stage 0 + erosion, one warp per 240-column strip and run
//                 of rows of one frame, no block barriers (described below);
//                 writes the eroded mask and the candidate mask
//   stream_wide   the same outputs with 64-bit sums, for the rare runs that
//                 hold a valid pixel too large for the exact 32-bit sums
//   mask_sums, mask_list
//                 the candidates as an ascending list (two scans of the mask)
//   seg_stage2    the background-only Poisson test at each candidate, exact;
//                 clears the failures from the mask, which is then the final
//                 strong-pixel mask
//   pass_sums, pass_scatter
//                 the passing candidates compacted in list order: the signal
//                 list, ascending by index
//   mask_prefix   (when asked for) each final-mask word's list position

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <mutex>

#include "sf_common.cuh"
#include "sf_scan.cuh"
#include "sf_stream.cuh"

namespace sf {

// Packed exact sums: the window's masked-pixel count in the top bits (enough
// for the largest window, (2K+1)^2 pixels), the sum of the valid ones in the
// rest.
constexpr int pack_shift(int K) {
  return (2 * K + 1) * (2 * K + 1) < 32 ? 27 : (2 * K + 1) * (2 * K + 1) < 64 ? 26 : 25;
}

// Fixed-point bits of the decision constants (sf_stream.cuh).
constexpr int kDecShift = 8;

// ---------------------------------------------------------------------------
// Stage 0 and the erosion, one warp per (frame, strip, run of rows).
//
// Lane l owns the 8 columns [X + 8 l, X + 8 l + 8) and walks down the run one
// pixel row at a time with no block barrier: it loads the 16 pixels
// [X + 8 l - 4, X + 8 l + 12) of the row (four 16-byte loads, the next row's
// prefetched), takes its 8 row sums of 2K+1 columns in registers (masked
// count and sum packed as m << PS | S, exact; p^2 exact in 32 bits), and
// carries 8 column sums down in registers; the row sum leaving the window
// comes back from a small per-lane ring in shared memory. Each new stage-0
// row gives 8 decisions (sf_stream.cuh) from two 64-bit bounds per window,
// with the constants for the window's masked count from a small table; the
// rare windows between the bounds are decided exactly, out of line. The
// common path has no divergent branch: on this SIMT machine a rarely taken
// per-lane branch still costs the whole warp its schedule, so masked pixels
// are folded in by selects rather than a separate path. The decisions are kept as
// 8-bit chunks in a 64-bit history; the erosion ANDs
// 2E+1 chunks vertically, then across columns with the neighbouring lanes'
// chunks (two shuffles). Lanes 0 and 31 are halo: they feed their
// neighbours' erosion and write nothing, so a warp writes 240 columns.
// ---------------------------------------------------------------------------

constexpr int kSegLanes = 32;
constexpr int kSegOut = 240;          // output columns per warp
constexpr int kSegWarps = 2;          // warps per block

template <int K> struct SegG {
  static constexpr int E = K - 1;
  static constexpr int R1 = 2 * K - 1;
  static constexpr int W0 = 2 * K + 1;
  static constexpr int N0 = W0 * W0;
  // Rows before a run's first output row: the windows fill (2K) and the
  // erosion's decision rows (2E).
  static constexpr int PRO = 2 * K + 2 * E;
  static constexpr uint32_t PS = pack_shift(K);
  static constexpr uint32_t MASK = (1u << PS) - 1u;
  // Blocks per SM that shared memory and registers allow (the ring grows
  // with K).
  static constexpr int OCC = K == 2 ? 8 : K == 3 ? 7 : 5;
  static_assert(R1 <= 7, "eight rows of history");
  static_assert(PRO == R1 + 2 * K - 1, "the first steady row outputs the run's first row");
};

template <int K> struct SegSmem {
  using G = SegG<K>;
  // ring[warp][slot][quad][lane] : uint4 = 4 of the 16 row sums
  uint4 ring[kSegWarps][G::W0][4][kSegLanes];
  // Decision constants by masked count m (window count N0 - m):
  // {2^8 n or 0, clo, chi, 0}.
  uint4 tab[G::N0 + 1];
};

__device__ __forceinline__ void seg_load(const uint32_t *__restrict__ image, int height, int width,
                                         bool interior, int cx, int p, uint32_t v[16]) {
  if (p < 0 || p >= height) {
#pragma unroll
    for (int i = 0; i < 16; i++)
      v[i] = 0xFFFFFFFFu;
    return;
  }
  const uint32_t *row = image + (size_t)p * width + (cx - 4);
  if (interior) {
#pragma unroll
    for (int f = 0; f < 4; f++) {
      const uint4 t = __ldg(reinterpret_cast<const uint4 *>(row) + f);
      v[4 * f] = t.x, v[4 * f + 1] = t.y, v[4 * f + 2] = t.z, v[4 * f + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const int gx = cx - 4 + i;
      v[i] = (gx >= 0 && gx < width) ? __ldg(row + i) : 0xFFFFFFFFu;
    }
  }
}

// What one warp's run writes to, resolved once per warp.
struct SegRun {
  const uint32_t *image;
  uint8_t *scr1_bytes, *final_bytes, *amb_bytes;
  uint32_t *wide_ctr;
  uint4 *wide_list;
  int frame, height, width, bytes_per_row;
  int X, cx, ra, rb, p0, warp, lane;
  bool writer;
  uint32_t inside8;
};

// Everything a lane carries from row to row.
template <int K> struct SegState {
  uint32_t vns[8], vq[8];
  unsigned long long hval, hs0;
  int slot;
};

// The two bounds of one window (sf_stream.cuh), branch-free:
// maybe = 2^8 n Q > S (2^8 S + clo), sure = 2^8 n Q >= S (2^8 S + chi) + 2^9.
__device__ __forceinline__ void seg_bounds(uint32_t S, uint32_t Q, uint32_t nk, uint32_t clo,
                                           uint32_t chi, bool *maybe, bool *sure) {
  const unsigned long long L = (unsigned long long)Q * nk;
  const uint32_t tl = (S << kDecShift) + clo, th = (S << kDecShift) + chi;
  *maybe = L > (unsigned long long)S * tl;
  *sure = L >= (unsigned long long)S * th + (2ull << kDecShift);
}

// One pixel row p for this lane. Steady rows (every row past a run's first
// PRO) output an eroded row; the first PRO rows only fill the windows and the
// decision history. Nothing here branches on the data: a row holding a pixel
// too large for the 32-bit sums returns true (the warp hands the rest of its
// run to the 64-bit path when it is done; what it writes past that row is
// rewritten there), and the windows between the two bounds are taken as
// signal here and recorded in the ambiguous mask for amb_fix.
template <int K, bool kSteady>
__device__ __forceinline__ bool seg_row(SegSmem<K> &s, SegState<K> &st, const uint32_t raw[16],
                                        int p, const SegRun &r, const StreamTables &T) {
  using G = SegG<K>;
  constexpr int o = 4 - K;               // first of the 8 + 2K pixels used
  constexpr int NP = 8 + 2 * K;
  const uint32_t narrow = T.narrow_max;

  // The pixels the row sums use, as masked-count << PS | value and value^2,
  // without a branch: u = v + 2 sends the masked sentinels to 0 and 1, a
  // masked pixel packs as a count bit alone, and its square (2^PS)^2 wraps
  // to 0. A valid pixel at or above narrow_max ends the narrow sums.
  uint32_t ns[16], q[16], valid8 = 0;
  bool wide;
  {
    uint32_t u[16];
#pragma unroll
    for (int i = o; i < o + NP; i++)
      u[i] = raw[i] + 2u;
    uint32_t m4[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      uint32_t a = 0;
#pragma unroll
      for (int i = o + j; i < o + NP; i += 4)
        a = max(a, u[i]);
      m4[j] = a;
    }
    wide = max(max(m4[0], m4[1]), max(m4[2], m4[3])) >= narrow + 2u;
#pragma unroll
    for (int i = o; i < o + NP; i++) {
      const bool ok = u[i] >= 2u;
      ns[i] = ok ? raw[i] : (1u << G::PS);
      q[i] = ns[i] * ns[i];
      if (i >= 4 && i < 12 && ok)
        valid8 |= 1u << (i - 4);
    }
  }
  const bool wide_row = __any_sync(0xffffffffu, wide);
  st.hval = (st.hval << 8) | valid8;

  // Row sums of 2K + 1 columns for the 8 columns, as two sliding chains.
  uint32_t hn[8], hq[8];
#pragma unroll
  for (int h = 0; h < 8; h += 4) {
    uint32_t a = 0, b = 0;
#pragma unroll
    for (int d = 0; d < G::W0; d++) {
      a += ns[o + h + d];
      b += q[o + h + d];
    }
    hn[h] = a;
    hq[h] = b;
#pragma unroll
    for (int c = h + 1; c < h + 4; c++) {
      a += ns[o + c + 2 * K] - ns[o + c - 1];
      b += q[o + c + 2 * K] - q[o + c - 1];
      hn[c] = a;
      hq[c] = b;
    }
  }

  // Column sums: the row sums of W0 rows ago come back from the ring.
  {
    uint4 *rg = &s.ring[r.warp][st.slot][0][r.lane];
    const uint4 l0 = rg[0], l1 = rg[32], l2 = rg[64], l3 = rg[96];
    const uint32_t ln[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
    const uint32_t lq[8] = {l2.x, l2.y, l2.z, l2.w, l3.x, l3.y, l3.z, l3.w};
#pragma unroll
    for (int c = 0; c < 8; c++) {
      st.vns[c] += hn[c] - ln[c];
      st.vq[c] += hq[c] - lq[c];
    }
    rg[0] = make_uint4(hn[0], hn[1], hn[2], hn[3]);
    rg[32] = make_uint4(hn[4], hn[5], hn[6], hn[7]);
    rg[64] = make_uint4(hq[0], hq[1], hq[2], hq[3]);
    rg[96] = make_uint4(hq[4], hq[5], hq[6], hq[7]);
    st.slot = st.slot + 1 == G::W0 ? 0 : st.slot + 1;
  }
  if (!kSteady && p < r.p0 + 2 * K)
    return wide_row;  // the column sums are not yet full windows (warp-uniform)

  // Stage-0 row p - K: eight decisions, maybe/sure bits without a branch
  // (the constants by masked count come from a small table; nearly every
  // lane reads the same entry); masked pixels are set.
  const uint32_t vrow = (uint32_t)(st.hval >> (8 * K)) & 0xFFu;
  uint32_t maybe8 = 0, sure8 = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    // The masked count is at most N0 while the sums are exact; past a
    // too-large pixel they are not, and the clamp keeps the read in bounds.
    const uint4 t = s.tab[min(st.vns[c] >> G::PS, (uint32_t)G::N0)];
    bool mb, su;
    seg_bounds(st.vns[c] & G::MASK, st.vq[c], t.x, t.y, t.z, &mb, &su);
    maybe8 |= mb ? 1u << c : 0u;
    sure8 |= su ? 1u << c : 0u;
  }
  const uint32_t amb8 = maybe8 & ~sure8 & vrow;
  const uint32_t s8 = (~vrow | sure8 | amb8) & 0xFFu;
  const int d = p - K;  // the decision row; each run records its own rows'
  if (r.writer && d >= r.ra && d < r.rb)
    r.amb_bytes[(size_t)d * r.bytes_per_row + (r.cx >> 3)] = (uint8_t)amb8;
  st.hs0 = (st.hs0 << 8) | s8;
  if (!kSteady)
    return wide_row;  // the erosion needs 2E more decision rows

  // Erosion of row p - R1: vertical AND of 2E + 1 chunks, then across columns
  // with the neighbours' chunks.
  uint32_t v8 = 0xFFu;
#pragma unroll
  for (int b = 0; b <= 2 * G::E; b++)
    v8 &= (uint32_t)(st.hs0 >> (8 * b)) & 0xFFu;
  const uint32_t left = __shfl_up_sync(0xffffffffu, v8, 1);
  const uint32_t right = __shfl_down_sync(0xffffffffu, v8, 1);
  const uint32_t all = (right << 16) | (v8 << 8) | left;
  uint32_t h8 = 0xFFu;
#pragma unroll
  for (int d = -G::E; d <= G::E; d++)
    h8 &= (all >> (8 + d)) & 0xFFu;
  const uint32_t masked8 = ~(uint32_t)(st.hval >> (8 * G::R1)) & 0xFFu;
  const uint32_t scr1 = (h8 | masked8) & r.inside8;
  const int re = p - G::R1;  // within [ra, rb) on every steady row
  if (r.writer) {
    // Candidates: eroded and not masked. The final mask starts as them and
    // stage 2 clears those that fail (the global threshold among them).
    const size_t at = (size_t)re * r.bytes_per_row + (r.cx >> 3);
    r.scr1_bytes[at] = (uint8_t)scr1;
    r.final_bytes[at] = (uint8_t)(scr1 & ~masked8);
  }
  return wide_row;
}

template <int K>
__global__ void __launch_bounds__(kSegWarps * 32, SegG<K>::OCC)
seg_stage01(const __grid_constant__ FramePtrs F, int nframes, int height, int width, int vec,
            int nstrips, int nruns, int run_rows, const __grid_constant__ LaunchParams P,
            const __grid_constant__ StreamTables T, uint8_t *__restrict__ scr1_bytes,
            uint8_t *__restrict__ final_bytes, uint8_t *__restrict__ amb_bytes, size_t mask_bytes,
            uint32_t *__restrict__ counters, uint4 *__restrict__ wide_list) {
  using G = SegG<K>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SegSmem<K> &s = *reinterpret_cast<SegSmem<K> *>(smem_raw);
  for (int m = threadIdx.x; m <= G::N0; m += blockDim.x)
    s.tab[m] = make_uint4(T.nk[G::N0 - m], T.clo[G::N0 - m], T.chi[G::N0 - m], 0u);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gw = blockIdx.x * kSegWarps + warp;
  const int sx = gw % nstrips, t = gw / nstrips;
  const int ry = t % nruns, f = t / nruns;
  if (f >= nframes)
    return;  // whole warp
  SegRun r;
  r.frame = f;
  r.image = F.image[f];
  r.height = height;
  r.width = width;
  r.bytes_per_row = ((width + 31) >> 5) * 4;
  r.scr1_bytes = scr1_bytes + (size_t)f * mask_bytes;
  r.final_bytes = final_bytes + (size_t)f * mask_bytes;
  r.amb_bytes = amb_bytes + (size_t)f * mask_bytes;
  r.wide_ctr = counters + kCtrWide;
  r.wide_list = wide_list;
  r.X = kSegOut * sx - 8;
  r.cx = r.X + 8 * lane;
  r.ra = ry * run_rows;
  r.rb = min(height, r.ra + run_rows);
  r.p0 = r.ra - G::R1;
  r.warp = warp;
  r.lane = lane;
  r.writer = lane >= 1 && lane <= 30 && r.cx < r.bytes_per_row * 8;
  // Bits of this lane's columns that lie inside the frame.
  r.inside8 = r.cx >= width ? 0u : (r.cx + 8 <= width ? 0xFFu : ((1u << (width - r.cx)) - 1u));
  const bool interior = vec && r.cx - 4 >= 0 && r.cx + 12 <= width;

#pragma unroll
  for (int sl = 0; sl < G::W0; sl++)
#pragma unroll
    for (int qd = 0; qd < 4; qd++)
      s.ring[warp][sl][qd][lane] = make_uint4(0u, 0u, 0u, 0u);
  __syncwarp();

  SegState<K> st;
#pragma unroll
  for (int c = 0; c < 8; c++)
    st.vns[c] = st.vq[c] = 0u;
  st.hval = st.hs0 = 0ull;
  st.slot = 0;

  // Pixel rows [p0, p1): the first PRO fill the windows and the history,
  // then every row outputs one eroded row (two per pass, the loads of the
  // next row prefetched into the other buffer).
  const int p1 = r.rb + G::R1;
  int first_wide = INT_MAX;
  for (int p = r.p0; p < r.p0 + G::PRO; p++) {
    uint32_t v[16];
    seg_load(r.image, height, width, interior, r.cx, p, v);
    if (seg_row<K, false>(s, st, v, p, r, T))
      first_wide = min(first_wide, p);
  }
  {
    uint32_t A[16], B[16];
    int p = r.p0 + G::PRO;
    seg_load(r.image, height, width, interior, r.cx, p, A);
    for (; p < p1; p += 2) {
      if (p + 1 < p1)
        seg_load(r.image, height, width, interior, r.cx, p + 1, B);
      if (seg_row<K, true>(s, st, A, p, r, T))
        first_wide = min(first_wide, p);
      if (p + 1 >= p1)
        break;
      if (p + 2 < p1)
        seg_load(r.image, height, width, interior, r.cx, p + 2, A);
      if (seg_row<K, true>(s, st, B, p + 1, r, T))
        first_wide = min(first_wide, p + 1);
    }
  }
  if (first_wide != INT_MAX && lane == 0) {
    // From the first row with a too-large pixel on, the 64-bit path redoes
    // the eroded rows [yb, rb) (their windows reach that row) and clears the
    // ambiguous records of the decision rows [dz, rb) written from bad sums.
    const uint32_t k = atomicAdd(r.wide_ctr, 1u);
    // Up to the end of the row's last mask word: the columns past the frame
    // are written as zeros there, as the lanes here would have.
    const int xb = max(0, r.X + 8), xe = min(r.bytes_per_row * 8, r.X + 8 + kSegOut);
    const int yb = max(r.ra, first_wide - G::R1), dz = max(r.ra, first_wide - K);
    r.wide_list[2 * k] = make_uint4((uint32_t)xb, (uint32_t)xe, (uint32_t)yb, (uint32_t)r.rb);
    r.wide_list[2 * k + 1] = make_uint4((uint32_t)r.frame, (uint32_t)dz, 0u, 0u);
  }
}

// ---------------------------------------------------------------------------
// Runs holding a pixel too large for the exact 32-bit sums: 32 x 32 tiles of
// the eroded mask with 64-bit sums, for the columns [xb, xe) and rows
// [yb, ye) of the frame a warp handed over.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(256)
stream_wide(const __grid_constant__ FramePtrs F, int height, int width, int run_rows,
            const __grid_constant__ LaunchParams P, uint8_t *__restrict__ scr1_all,
            uint8_t *__restrict__ final_all, uint8_t *__restrict__ amb_all, size_t mask_bytes,
            uint32_t *__restrict__ counters, const uint4 *__restrict__ wide_list) {
  constexpr int E = K - 1, R1 = 2 * K - 1;
  constexpr int TS = 32, IW = TS + 2 * R1, S0 = IW - 2 * K;
  __shared__ uint32_t pix[IW][IW];
  __shared__ unsigned long long hS[IW][S0], hQ[IW][S0];
  __shared__ uint8_t hN[IW][S0];
  __shared__ uint8_t scr0[S0][S0];
  __shared__ uint32_t rlo[kMaxN0 + 1], rhi[kMaxN0 + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int bytes_per_row = ((width + 31) >> 5) * 4;
  for (int i = tid; i <= kMaxN0; i += blockDim.x) {
    rlo[i] = P.root_lo[i];
    rhi[i] = P.root_hi[i];
  }
  const uint32_t nwide = counters[kCtrWide];
  constexpr int TPS = (kSegOut + TS - 1) / TS;  // tile columns per entry
  const int TPR = (run_rows + TS - 1) / TS;      // tile rows per entry
  for (uint32_t item = blockIdx.x; item < nwide * TPS * TPR; item += gridDim.x) {
    const uint32_t k = item / (TPS * TPR);
    const uint4 w = wide_list[2 * k];
    const int f = (int)wide_list[2 * k + 1].x, dz = (int)wide_list[2 * k + 1].y;
    uint8_t *amb_bytes = amb_all + (size_t)f * mask_bytes;
    const uint32_t *image = F.image[f];
    uint8_t *scr1_bytes = scr1_all + (size_t)f * mask_bytes;
    uint8_t *final_bytes = final_all + (size_t)f * mask_bytes;
    const int rem = (int)(item % (TPS * TPR));
    const int tcol = rem % TPS, trow = rem / TPS;
    const int xb = (int)w.x, xe = (int)w.y, yb = (int)w.z, ye = (int)w.w;
    const int tx0 = xb + tcol * TS, ty0 = yb + trow * TS;
    if (ty0 >= ye || tx0 >= xe)
      continue;  // block-uniform
    const int ty1 = min(ye, ty0 + TS);
    __syncthreads();
    for (int i = tid; i < IW * IW; i += blockDim.x) {
      const int r = i / IW, c = i - r * IW;
      const int gy = ty0 - R1 + r, gx = tx0 - R1 + c;
      pix[r][c] = (gy >= 0 && gy < height && gx >= 0 && gx < width)
                      ? image[(size_t)gy * width + gx] : 0xFFFFFFFFu;
    }
    __syncthreads();
    for (int i = tid; i < IW * S0; i += blockDim.x) {
      const int r = i / S0, c = i - r * S0;
      uint32_t n = 0;
      unsigned long long S = 0, Q = 0;
      for (int d = 0; d <= 2 * K; d++) {
        const uint32_t v = pix[r][c + d];
        if (v < 0xFFFFFFFEu) {
          n++;
          S += v;
          Q += (unsigned long long)v * v;
        }
      }
      hN[r][c] = (uint8_t)n;
      hS[r][c] = S;
      hQ[r][c] = Q;
    }
    __syncthreads();
    for (int i = tid; i < S0 * S0; i += blockDim.x) {
      const int r = i / S0, c = i - r * S0;
      uint32_t n = 0;
      unsigned long long S = 0, Q = 0;
      for (int d = 0; d <= 2 * K; d++) {
        n += hN[r + d][c];
        S += hS[r + d][c];
        Q += hQ[r + d][c];
      }
      const bool sig = stage0_u32(n, S, Q, P, rlo, rhi);
      scr0[r][c] = (sig || pix[r + K][c + K] >= 0xFFFFFFFEu) ? 1 : 0;
    }
    __syncthreads();
    for (int r = warp; r < TS; r += blockDim.x >> 5) {
      const int gy = ty0 + r, c = lane, gx = tx0 + c;
      const uint32_t v = pix[r + R1][c + R1];
      bool m = true;
      if (v < 0xFFFFFFFEu) {
        m = scr0[r + E][c + E];
        for (int dr = 0; dr <= 2 * E && m; dr++)
          for (int dc = 0; dc <= 2 * E; dc++)
            if (!scr0[r + dr][c + dc]) {
              m = false;
              break;
            }
      }
      const bool b = gy < ty1 && gx < min(xe, width) && m;
      const uint32_t word = __ballot_sync(0xffffffffu, b);
      const unsigned cm = __ballot_sync(0xffffffffu, b && v < 0xFFFFFFFEu);
      if (gy < ty1 && lane < 4) {
        const int bx = tx0 + 8 * lane;
        if (bx < xe && (bx >> 3) < bytes_per_row) {
          scr1_bytes[(size_t)gy * bytes_per_row + (bx >> 3)] = (uint8_t)(word >> (8 * lane));
          final_bytes[(size_t)gy * bytes_per_row + (bx >> 3)] = (uint8_t)(cm >> (8 * lane));
          if (gy >= dz)
            amb_bytes[(size_t)gy * bytes_per_row + (bx >> 3)] = 0;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// The windows between the two bounds (the ambiguous mask): each is decided
// exactly from its 64-bit sums (src/spots/dext.cc:99-109, sf_common.cuh). The
// first pass took each as signal; where it is not, its (2E+1)^2 neighbourhood
// cannot survive the erosion (an AND of the stage-0 bits), so every valid
// pixel there leaves the eroded and candidate masks. A clearing is true of
// the frame whatever else was decided, so the order of the fixes, and any
// ambiguous record left by rows the 64-bit path rewrote, do not matter.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(256)
amb_fix(const __grid_constant__ FramePtrs F, int height, int width,
        const __grid_constant__ LaunchParams P, const uint32_t *__restrict__ amb_all,
        uint32_t *__restrict__ scr1_all, uint32_t *__restrict__ final_all, size_t words) {
  constexpr int E = K - 1;
  const int f = blockIdx.y;
  const uint32_t *image = F.image[f];
  const uint32_t *amb = amb_all + (size_t)f * words;
  uint32_t *scr1 = scr1_all + (size_t)f * words;
  uint32_t *fin = final_all + (size_t)f * words;
  const uint32_t wpr = ((uint32_t)width + 31u) >> 5;
  // One thread per mask word: the scan runs at memory speed, and the rare
  // set bits are handled where they are found.
  const size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w < words) {
    uint32_t bits = amb[w];
    const int y = (int)(w / wpr);
    const int x0 = (int)(w - (size_t)y * wpr) * 32;
    while (bits) {
      const int x = x0 + __ffs(bits) - 1;
      bits &= bits - 1u;
      uint32_t n = 0;
      unsigned long long S = 0, Q = 0;
      for (int dy = -K; dy <= K; dy++) {
        const int yy = y + dy;
        if (yy < 0 || yy >= height)
          continue;
        for (int dx = -K; dx <= K; dx++) {
          const int xx = x + dx;
          if (xx < 0 || xx >= width)
            continue;
          const uint32_t v = __ldg(image + (size_t)yy * width + xx);
          if (v < 0xFFFFFFFEu) {
            n++;
            S += v;
            Q += (unsigned long long)v * v;
          }
        }
      }
      if (stage0_u32(n, S, Q, P, P.root_lo, P.root_hi))
        continue;
      for (int dy = -E; dy <= E; dy++) {
        const int yy = y + dy;
        if (yy < 0 || yy >= height)
          continue;
        for (int dx = -E; dx <= E; dx++) {
          const int xx = x + dx;
          if (xx < 0 || xx >= width || __ldg(image + (size_t)yy * width + xx) >= 0xFFFFFFFEu)
            continue;
          const size_t at = (size_t)yy * wpr + (xx >> 5);
          const uint32_t keep = ~(1u << (xx & 31));
          atomicAnd(scr1 + at, keep);
          atomicAnd(fin + at, keep);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// The candidate list: the set bits of the candidate mask (the final mask as
// the first pass wrote it), ascending, from two scans over the mask words.
// Every kernel below runs on a (block, frame) grid.
// ---------------------------------------------------------------------------
constexpr int kScanT = 256;                    // threads of a scan block
constexpr int kScanPer = 8;                    // consecutive items per thread
constexpr int kScanChunk = kScanT * kScanPer;  // items per block pass

// This block's share [lo, hi) of a frame's n items, in whole passes.
__device__ __forceinline__ void chunk_of(size_t n, size_t *lo, size_t *hi) {
  size_t chunk = (n + gridDim.x - 1) / gridDim.x;
  chunk = (chunk + kScanChunk - 1) / kScanChunk * kScanChunk;
  *lo = min(n, (size_t)blockIdx.x * chunk);
  *hi = min(n, *lo + chunk);
}

// Sum of the block's predecessors' counts in its frame, and the frame's
// total.
__device__ __forceinline__ uint32_t block_base(const uint32_t *__restrict__ block_sums,
                                               uint32_t *total) {
  __shared__ uint32_t s_base, s_total;
  if (threadIdx.x < 32) {
    const uint32_t *bs = block_sums + (size_t)blockIdx.y * gridDim.x;
    uint32_t b = 0, t = 0;
    for (uint32_t i = threadIdx.x; i < gridDim.x; i += 32) {
      const uint32_t v = bs[i];
      b += i < blockIdx.x ? v : 0u;
      t += v;
    }
    for (int o = 16; o; o >>= 1) {
      b += __shfl_xor_sync(0xffffffffu, b, o);
      t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    if (threadIdx.x == 0) {
      s_base = b;
      s_total = t;
    }
  }
  __syncthreads();
  *total = s_total;
  return s_base;
}

// Every item of [lo, hi) with its count's exclusive prefix (offset by
// carry): emit(i, item, position) for items that count.
template <typename V, class Load, class Count, class Emit>
__device__ __forceinline__ void scan_emit(size_t lo, size_t hi, uint32_t carry, Load load,
                                          Count count, Emit emit) {
  for (size_t base = lo; base < hi; base += kScanChunk) {
    const size_t i0 = base + (size_t)threadIdx.x * kScanPer;
    V v[kScanPer];
    uint32_t c[kScanPer], tot = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      const bool in = i0 + k < hi;
      v[k] = in ? load(i0 + k) : V();
      c[k] = in ? count(v[k]) : 0u;
      tot += c[k];
    }
    uint32_t t;
    uint32_t pos = carry + block_exclusive_scan(tot, &t);
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      if (c[k])
        emit(i0 + k, v[k], pos);
      pos += c[k];
    }
    carry += t;
  }
}

// A thread's kScanPer consecutive mask words from i0 (16-byte loads where
// the frame's words are 16-byte aligned and all 8 lie before hi).
__device__ __forceinline__ void load_words(const uint32_t *__restrict__ bits, size_t i0,
                                           size_t hi, bool vec, uint32_t w[kScanPer]) {
  static_assert(kScanPer == 8, "two 16-byte loads a thread");
  if (vec && i0 + kScanPer <= hi) {
    const uint4 a = __ldg(reinterpret_cast<const uint4 *>(bits + i0));
    const uint4 b = __ldg(reinterpret_cast<const uint4 *>(bits + i0 + 4));
    w[0] = a.x, w[1] = a.y, w[2] = a.z, w[3] = a.w;
    w[4] = b.x, w[5] = b.y, w[6] = b.z, w[7] = b.w;
    return;
  }
#pragma unroll
  for (int k = 0; k < kScanPer; k++)
    w[k] = i0 + k < hi ? bits[i0 + k] : 0u;
}

// A thread's kScanPer consecutive stage-2 results from i0 (16-byte loads,
// two results each, where the frame's results are 16-byte aligned and all 8
// lie before hi); zeros past hi.
__device__ __forceinline__ void load_res(const uint2 *__restrict__ res, size_t i0, size_t hi,
                                         bool vec, uint2 r[kScanPer]) {
  if (vec && i0 + kScanPer <= hi) {
    const uint4 *r4 = reinterpret_cast<const uint4 *>(res + i0);
#pragma unroll
    for (int k = 0; k < kScanPer / 2; k++) {
      const uint4 x = __ldg(r4 + k);
      r[2 * k] = make_uint2(x.x, x.y);
      r[2 * k + 1] = make_uint2(x.z, x.w);
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < kScanPer; k++)
    r[k] = i0 + k < hi ? res[i0 + k] : make_uint2(0u, 0u);
}

// Popcounts of the block's share of a frame's mask words.
__global__ void __launch_bounds__(kScanT)
mask_sums(const __grid_constant__ FramePtrs F, const uint32_t *__restrict__ bits_all, size_t words,
          uint32_t *__restrict__ block_sums) {
  const uint32_t *bits = bits_all + (size_t)blockIdx.y * words;
  const bool vec = reinterpret_cast<uintptr_t>(bits) % 16 == 0;
  size_t lo, hi;
  chunk_of(frame_words(F, blockIdx.y), &lo, &hi);
  uint32_t acc = 0;
  for (size_t base = lo; base < hi; base += kScanChunk) {
    uint32_t w[kScanPer];
    load_words(bits, base + (size_t)threadIdx.x * kScanPer, hi, vec, w);
#pragma unroll
    for (int k = 0; k < kScanPer; k++)
      acc += (uint32_t)__popc(w[k]);
  }
  uint32_t total;
  (void)block_exclusive_scan(acc, &total);
  if (threadIdx.x == 0)
    block_sums[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = total;
}

// The pixel index of every set bit of the block's share, in order.
__global__ void __launch_bounds__(kScanT)
mask_list(const uint32_t *__restrict__ bits_all, size_t words, int width,
          const uint32_t *__restrict__ block_sums, uint32_t *__restrict__ cand_all,
          uint32_t cand_cap, uint32_t *__restrict__ counters) {
  const int f = blockIdx.y;
  const uint32_t *bits = bits_all + (size_t)f * words;
  uint32_t *cand = cand_all + (size_t)f * cand_cap;
  uint32_t total;
  const uint32_t carry = block_base(block_sums, &total);
  if (blockIdx.x == 0 && threadIdx.x == 0)
    counters[kCtrBatch + (size_t)f * kCtrCount + kCtrCand] = total;
  const uint32_t wpr = ((uint32_t)width + 31u) >> 5;
  size_t lo, hi;
  chunk_of(words, &lo, &hi);
  scan_emit<uint32_t>(
      lo, hi, carry, [&](size_t w) { return bits[w]; },
      [](uint32_t word) { return (uint32_t)__popc(word); },
      [&](size_t w, uint32_t word, uint32_t pos) {
        const uint32_t row = (uint32_t)w / wpr;
        const uint32_t first = row * (uint32_t)width + ((uint32_t)w - row * wpr) * 32u;
        while (word) {
          const int b = __ffs(word) - 1;
          word &= word - 1u;
          if (pos < cand_cap)
            cand[pos] = first + (uint32_t)b;
          pos++;
        }
      });
}

// ---------------------------------------------------------------------------
// Stage 2 at the candidates, four lanes to a candidate: each lane sums a
// quarter of the (2K + 5) rows of the clipped window, two shuffles add them.
// Away from the frame's edges a lane reads a window row as four aligned
// 16-byte loads (the 16 columns from the window's first column rounded down
// to a multiple of 4) and the eroded-mask bits over them as a 64-bit pair,
// every row's loads issued together. The result of candidate i goes to
// res[i] (the background's bits; the population, and the pass bit at 16),
// and a candidate that fails is cleared from the final mask.
// ---------------------------------------------------------------------------
// k32: every valid pixel of the frame is below 2^24 (no run needed the 64-bit
// path), so a window's background sum (at most 169 of them) fits 32 bits.
template <int K, bool k32>
__device__ __forceinline__ void s2_window(const uint32_t *__restrict__ image,
                                          const uint32_t *__restrict__ scr1_words, int height,
                                          int width, int wpr, int vec, int sub, int y, int x,
                                          uint32_t *n_out, unsigned long long *S_out) {
  constexpr int K2 = K + 2, WW = 2 * K2 + 1, ROWS = (WW + 3) / 4;
  static_assert(WW + 3 <= 16, "a window row fits four aligned 16-byte loads");
  uint32_t n = 0;
  unsigned long long S = 0;
  const int xa = (x - K2) & ~3;
  if (vec && x - K2 >= 0 && xa + 16 <= width) {
    const int off = (x - K2) - xa;
    const int w0 = xa >> 5, sh = xa & 31;
    const uint32_t win = ((1u << WW) - 1u) << off;
    // Rows off the frame (or past the window) read a clamped row and count
    // nothing.
    uint32_t bgs[ROWS];
    uint4 t[ROWS][4];
#pragma unroll
    for (int k = 0; k < ROWS; k++) {
      const int dy = -K2 + sub + 4 * k;
      const int yy = y + dy;
      const bool in = dy <= K2 && yy >= 0 && yy < height;
      const int yc = min(max(yy, 0), height - 1);
      const uint4 *row = reinterpret_cast<const uint4 *>(image + (size_t)yc * width + xa);
      const uint32_t *brow = scr1_words + (size_t)yc * wpr;
      const uint32_t b0 = __ldg(brow + w0);
      const uint32_t b1 = (w0 + 1 < wpr) ? __ldg(brow + w0 + 1) : 0u;
#pragma unroll
      for (int q = 0; q < 4; q++)
        t[k][q] = __ldg(row + q);
      const unsigned long long both = (unsigned long long)b0 | ((unsigned long long)b1 << 32);
      bgs[k] = in ? (~(uint32_t)(both >> sh) & win) : 0u;
    }
#pragma unroll
    for (int k = 0; k < ROWS; k++) {
      const uint32_t bg = bgs[k];
      const uint32_t v[16] = {t[k][0].x, t[k][0].y, t[k][0].z, t[k][0].w,
                              t[k][1].x, t[k][1].y, t[k][1].z, t[k][1].w,
                              t[k][2].x, t[k][2].y, t[k][2].z, t[k][2].w,
                              t[k][3].x, t[k][3].y, t[k][3].z, t[k][3].w};
      // Not in the eroded mask, so valid (masked pixels are in it).
      n += __popc(bg);
      if (k32) {
        uint32_t s32 = 0;
#pragma unroll
        for (int d = 0; d < 16; d++)
          s32 += ((bg >> d) & 1u) ? v[d] : 0u;
        S += s32;
      } else {
#pragma unroll
        for (int d = 0; d < 16; d++)
          S += ((bg >> d) & 1u) ? v[d] : 0u;
      }
    }
  } else {
    const int xlo = max(0, x - K2), xhi = min(width - 1, x + K2);
    const int w0 = xlo >> 5;
#pragma unroll
    for (int k = 0; k < ROWS; k++) {
      const int dy = -K2 + sub + 4 * k;
      const int yy = y + dy;
      if (dy > K2 || yy < 0 || yy >= height)
        continue;
      const uint32_t *row = image + (size_t)yy * width;
      const uint32_t *brow = scr1_words + (size_t)yy * wpr;
      const unsigned long long both =
          (unsigned long long)__ldg(brow + w0) |
          ((w0 + 1 < wpr) ? ((unsigned long long)__ldg(brow + w0 + 1) << 32) : 0ull);
      const unsigned long long bgb = ~(both >> (xlo - (w0 << 5)));
#pragma unroll
      for (int d = 0; d < WW; d++)
        if (xlo + d <= xhi && ((bgb >> d) & 1ull)) {
          n++;
          S += __ldg(row + xlo + d);
        }
    }
  }
  *n_out = n;
  *S_out = S;
}

template <int K>
__global__ void __launch_bounds__(256)
seg_stage2(const __grid_constant__ FramePtrs F, int height, int width, int vec,
           const __grid_constant__ LaunchParams P, const uint32_t *__restrict__ scr1_all,
           uint32_t *__restrict__ final_all, size_t words, const uint32_t *__restrict__ cand_all,
           uint32_t cand_cap, const uint32_t *__restrict__ counters, uint2 *__restrict__ res_all) {
  const int f = blockIdx.y;
  const uint32_t *image = F.image[f];
  const uint32_t *scr1_words = scr1_all + (size_t)f * words;
  uint32_t *final_words = final_all + (size_t)f * words;
  const uint32_t *cand = cand_all + (size_t)f * cand_cap;
  uint2 *res = res_all + (size_t)f * cand_cap;
  const int wpr = (width + 31) >> 5;
  const uint32_t nc = min(counters[kCtrBatch + (size_t)f * kCtrCount + kCtrCand], cand_cap);
  // No run of the batch met a valid pixel at or above the narrow bound.
  const bool narrow = counters[kCtrWide] == 0 &&
                     counters[kCtrBatch + (size_t)f * kCtrCount + kCtrWideFrame] == 0;
  const int lane = threadIdx.x & 31, sub = lane & 3;
  const uint32_t per_pass = (gridDim.x * blockDim.x) >> 2;
  for (uint32_t base = (blockIdx.x * blockDim.x) >> 2; base < nc; base += per_pass) {
    const uint32_t i = base + (threadIdx.x >> 2);
    const bool live = i < nc;
    uint32_t idx = 0, p = 0, n = 0;
    unsigned long long S = 0;
    int y = 0, x = 0;
    if (live) {
      idx = cand[i];
      y = (int)(idx / (uint32_t)width);
      x = (int)(idx - (uint32_t)y * (uint32_t)width);
      p = __ldg(image + idx);
      if (narrow)
        s2_window<K, true>(image, scr1_words, height, width, wpr, vec, sub, y, x, &n, &S);
      else
        s2_window<K, false>(image, scr1_words, height, width, wpr, vec, sub, y, x, &n, &S);
    }
    n += __shfl_xor_sync(0xffffffffu, n, 1);
    S += __shfl_xor_sync(0xffffffffu, S, 1);
    n += __shfl_xor_sync(0xffffffffu, n, 2);
    S += __shfl_xor_sync(0xffffffffu, S, 2);
    if (live && sub == 0) {
      float bg = 0.0f;
      // dext.cc:205: only pixels above the global threshold are tested.
      const bool sig = (uint64_t)p >= P.p_min && stage2_u32(p, n, S, P, &bg);
      res[i] = make_uint2(__float_as_uint(bg), n | (sig ? 1u << 16 : 0u));
      if (!sig)
        atomicAnd(&final_words[(size_t)y * wpr + (x >> 5)], ~(1u << (x & 31)));
    }
  }
}

// ---------------------------------------------------------------------------
// The ordered list: the passing candidates compacted in list order, which is
// ascending pixel order (src/spots/dext.cc:212-220 emits in scan order).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kScanT)
pass_sums(const __grid_constant__ FramePtrs F, const uint2 *__restrict__ res_all, uint32_t cand_cap,
          const uint32_t *__restrict__ counters, uint32_t *__restrict__ block_sums,
          const uint32_t *__restrict__ cand_all, uint32_t *__restrict__ final_all, size_t words) {
  const int f = blockIdx.y;
  if (counters[kCtrFault]) {  // the stage-2 results are void: touch nothing
    if (threadIdx.x == 0)
      block_sums[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = 0;
    return;
  }
  const uint2 *res = res_all + (size_t)f * cand_cap;
  const uint32_t nc = min(counters[kCtrBatch + (size_t)f * kCtrCount + kCtrCand], cand_cap);
  // final_all given: the candidates that failed stage 2 leave the final mask
  // here (their stage 2 left it alone).
  const uint32_t *cand = cand_all + (size_t)f * cand_cap;
  uint32_t *fin = final_all ? final_all + (size_t)f * words : nullptr;
  const int width = F.w[f];
  const uint32_t wpr = ((uint32_t)width + 31u) >> 5;
  const bool vec = reinterpret_cast<uintptr_t>(res) % 16 == 0;
  size_t lo, hi;
  chunk_of(nc, &lo, &hi);
  uint32_t acc = 0;
  for (size_t base = lo; base < hi; base += kScanChunk) {
    const size_t i0 = base + (size_t)threadIdx.x * kScanPer;
    uint2 r[kScanPer];
    load_res(res, i0, hi, vec, r);
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      if (i0 + k >= hi)
        break;
      const uint32_t pass = (r[k].y >> 16) & 1u;
      if (fin && !pass) {
        const uint32_t idx = cand[i0 + k], y = idx / (uint32_t)width,
                       x = idx - y * (uint32_t)width;
        atomicAnd(fin + (size_t)y * wpr + (x >> 5), ~(1u << (x & 31)));
      }
      acc += pass;
    }
  }
  uint32_t total;
  (void)block_exclusive_scan(acc, &total);
  if (threadIdx.x == 0)
    block_sums[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = total;
}

template <typename Pix>
__global__ void __launch_bounds__(kScanT)
pass_scatter(const __grid_constant__ FramePtrs F, const uint32_t *__restrict__ cand_all,
             uint32_t cand_cap, const uint2 *__restrict__ res_all,
             const uint32_t *__restrict__ counters, const uint32_t *__restrict__ block_sums,
             sf_signal_pixel *__restrict__ out_all, size_t out_stride, uint32_t capacity,
             uint32_t *__restrict__ count_out) {
  const int f = blockIdx.y;
  if (counters[kCtrFault]) {  // a bounded device wait ran out: no list
    if (blockIdx.x == 0 && threadIdx.x == 0)
      count_out[f] = kCountFault;
    return;
  }
  const Pix *image = reinterpret_cast<const Pix *>(F.image[f]);
  const uint32_t *cand = cand_all + (size_t)f * cand_cap;
  const uint2 *res = res_all + (size_t)f * cand_cap;
  sf_signal_pixel *out = out_all + (size_t)f * out_stride;
  const uint32_t ncand = counters[kCtrBatch + (size_t)f * kCtrCount + kCtrCand];
  const uint32_t nc = min(ncand, cand_cap);
  uint32_t total;
  const uint32_t carry = block_base(block_sums, &total);
  if (blockIdx.x == 0 && threadIdx.x == 0)
    // The signal found; all ones if the candidate list overflowed, as for a
    // count above capacity (the list is then incomplete).
    count_out[f] = ncand > cand_cap ? 0xFFFFFFFFu : total;
  const bool vec = reinterpret_cast<uintptr_t>(res) % 16 == 0;
  const bool vec_c = reinterpret_cast<uintptr_t>(cand) % 16 == 0;
  size_t lo, hi;
  chunk_of(nc, &lo, &hi);
  uint32_t run = carry;
  for (size_t base = lo; base < hi; base += kScanChunk) {
    const size_t i0 = base + (size_t)threadIdx.x * kScanPer;
    uint2 r[kScanPer];
    load_res(res, i0, hi, vec, r);
    uint32_t idx[kScanPer];
    load_words(cand, i0, hi, vec_c, idx);
    // The passing pixels' values: every load in flight before the scan
    // (none waits for another).
    uint32_t c[kScanPer], val[kScanPer], tot = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      c[k] = i0 + k < hi ? (r[k].y >> 16) & 1u : 0u;
      val[k] = c[k] ? (uint32_t)__ldg(image + idx[k]) : 0u;
      tot += c[k];
    }
    uint32_t t;
    uint32_t pos = run + block_exclusive_scan(tot, &t);
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      if (c[k] && pos < capacity) {
        sf_signal_pixel rec;
        rec.index = idx[k];
        rec.value = val[k];
        rec.background = __uint_as_float(r[k].x);
        rec.population = (uint16_t)(r[k].y & 0xFFFFu);
        rec.reserved = 0;
        out[pos] = rec;
      }
      pos += c[k];
    }
    run += t;
  }
}

// Optional: per final-mask word, the list position of its first pixel.
__global__ void __launch_bounds__(kScanT)
mask_prefix(const __grid_constant__ FramePtrs F, const uint32_t *__restrict__ bits_all,
            size_t words, const uint32_t *__restrict__ block_sums,
            uint32_t *__restrict__ prefix_all, uint32_t *__restrict__ counters) {
  const int f = blockIdx.y;
  const uint32_t *bits = bits_all + (size_t)f * words;
  uint32_t *prefix = prefix_all + (size_t)f * words;
  uint32_t total;
  uint32_t carry = block_base(block_sums, &total);
  if (counters && blockIdx.x == 0 && threadIdx.x == 0)
    counters[kCtrBatch + (size_t)f * kCtrCount + kCtrCand] = total;  // the candidates
  const bool vec = reinterpret_cast<uintptr_t>(bits) % 16 == 0 &&
                   reinterpret_cast<uintptr_t>(prefix) % 16 == 0;
  size_t lo, hi;
  chunk_of(frame_words(F, f), &lo, &hi);
  for (size_t base = lo; base < hi; base += kScanChunk) {
    const size_t i0 = base + (size_t)threadIdx.x * kScanPer;
    uint32_t c[kScanPer], tot = 0;
    load_words(bits, i0, hi, vec, c);
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      c[k] = (uint32_t)__popc(c[k]);
      tot += c[k];
    }
    uint32_t t;
    uint32_t pos = carry + block_exclusive_scan(tot, &t);
    uint32_t p[kScanPer];
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      p[k] = pos;
      pos += c[k];
    }
    if (vec && i0 + kScanPer <= hi) {
      reinterpret_cast<uint4 *>(prefix + i0)[0] = make_uint4(p[0], p[1], p[2], p[3]);
      reinterpret_cast<uint4 *>(prefix + i0)[1] = make_uint4(p[4], p[5], p[6], p[7]);
    } else {
#pragma unroll
      for (int k = 0; k < kScanPer; k++)
        if (i0 + k < hi)
          prefix[i0 + k] = p[k];
    }
    carry += t;
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------

int device_sms() {
  static int cached = 0;
  if (cached)
    return cached;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms <= 0)
    return 152;  // not cached: asked again once a device answers
  cached = sms;
  return cached;
}

// Blocks per frame of the scan kernels: one per 2048 mask words (a scan
// block walks its share in two passes), at least one, never more than
// kOrderMaxBlocks over the batch.
constexpr int kOrderMaxBlocks = 8192;
static int order_bpf(int nframes, size_t words) {
  const long long want = (long long)((words + 2047) / 2048);
  return (int)std::max(1ll, std::min(want, (long long)(kOrderMaxBlocks / nframes)));
}

int stream_order_blocks() { return kOrderMaxBlocks; }

size_t stream_wide_entries(int h, int w, int nframes) {
  const size_t strips = (size_t)(w + kSegOut - 1) / kSegOut;
  const size_t runs = (size_t)(h + kMinRunRows - 1) / kMinRunRows;
  return (size_t)nframes * strips * runs;
}

SegGeometry seg_geometry(int h, int w, int nframes, int run_rows, int slots) {
  SegGeometry g;
  g.nstrips = (w + kSegOut - 1) / kSegOut;
  if (run_rows <= 0) {
    // As many runs as fit the resident warps in one wave: a second, partial
    // wave would double the kernel's time.
    const long long per = (long long)nframes * g.nstrips;
    const long long nruns = std::max(1ll, (long long)slots / per);
    run_rows = (int)((h + nruns - 1) / nruns);
  }
  g.run_rows = std::max(run_rows, kMinRunRows);
  g.nruns = (h + g.run_rows - 1) / g.run_rows;
  return g;
}

void make_stream_tables(const LaunchParams &P, StreamTables *T) {
  const int K = P.half;
  const int n0 = (2 * K + 1) * (2 * K + 1);
  const int ps = K == 2 ? pack_shift(2) : K == 3 ? pack_shift(3) : pack_shift(4);
  // Exact 32-bit sums: the count and sum packed below 2^32, and the window's
  // sum of p^2 below 2^32 (p < sqrt(2^32 / n0): 13107, 9362, 7282).
  const uint32_t by_pack = (uint32_t)(((1u << ps) - 1u) / (uint32_t)n0);
  uint32_t by_sq = (uint32_t)std::floor(std::sqrt(4294967295.0 / n0));
  while ((uint64_t)by_sq * by_sq * (uint64_t)n0 > 0xFFFFFFFFull)
    by_sq--;
  T->narrow_max = std::min(by_pack, by_sq + 1);
  for (int n = 0; n <= kMaxN0; n++) {
    const bool testable = n >= 1 && (uint32_t)n >= P.min_local && n <= n0;
    // 2^8 (n - 1 + sigma_b r_n) bracketed from r_n's 2^-20 floor and ceiling.
    const uint64_t sb = P.sigma_b_int;
    const uint64_t lo = testable ? (sb * P.root_lo[n]) >> (kRootShift - kDecShift) : 0;
    const uint64_t hi =
        testable ? (sb * P.root_hi[n] + ((1ull << (kRootShift - kDecShift)) - 1)) >>
                       (kRootShift - kDecShift)
                 : 0;
    const uint64_t base = testable ? (uint64_t)(n - 1) << kDecShift : 0;
    T->clo[n] = (uint32_t)(base + lo);
    T->chi[n] = (uint32_t)(base + hi);
    // nk 0 makes every such window "surely not" (0 <= S (2^8 S + clo)).
    T->nk[n] = testable ? (uint32_t)n << kDecShift : 0u;
  }
}

template <int K> static int seg_slots() {
  static int slots = 0;
  if (!slots) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, seg_stage01<K>, kSegWarps * 32,
                                                  sizeof(SegSmem<K>));
    slots = std::max(1, per) * kSegWarps * device_sms();
  }
  return slots;
}

template <int K>
static cudaError_t launch_stream_k(const FramePtrs &F, int nframes, int h, int w,
                                   const LaunchParams &P, const StreamBuffers &b, int run_rows,
                                   cudaStream_t stream, const StreamMarks *marks) {
  using S = SegSmem<K>;
  static std::once_flag configured;
  static cudaError_t config_error = cudaSuccess;
  std::call_once(configured, [] {
    config_error = cudaFuncSetAttribute(
        seg_stage01<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(S));
  });
  if (config_error != cudaSuccess)
    return config_error;
  StreamTables T;
  make_stream_tables(P, &T);
  int vec = 1;
  for (int f = 0; f < nframes; f++)
    if (F.w[f] % 4 != 0 || reinterpret_cast<uintptr_t>(F.image[f]) % 16 != 0)
      vec = 0;
  const int sms = device_sms();
  if (K == 3) {
    // The reference's window: the lattice bound and its exact check.
    const cudaError_t e = launch_lattice(F, nframes, h, w, vec, 4, P, T, b, run_rows, stream);
    if (e != cudaSuccess)
      return e;
  } else {
    const SegGeometry g = seg_geometry(h, w, nframes, run_rows, seg_slots<K>());
    const long long warps = (long long)nframes * g.nstrips * g.nruns;
    const size_t mask_bytes = b.words * sizeof(uint32_t);
    uint8_t *scr1 = reinterpret_cast<uint8_t *>(b.scr1);
    uint8_t *fin = reinterpret_cast<uint8_t *>(b.bits);
    uint8_t *amb = reinterpret_cast<uint8_t *>(b.amb);
    seg_stage01<K><<<(unsigned)((warps + kSegWarps - 1) / kSegWarps), kSegWarps * 32, sizeof(S),
                     stream>>>(F, nframes, h, w, vec, g.nstrips, g.nruns, g.run_rows, P, T, scr1,
                               fin, amb, mask_bytes, b.counters, b.wide);
    stream_wide<K><<<2 * sms, 256, 0, stream>>>(F, h, w, g.run_rows, P, scr1, fin, amb,
                                                 mask_bytes, b.counters, b.wide);
    amb_fix<K><<<dim3((unsigned)((b.words + 255) / 256), nframes), 256, 0, stream>>>(
        F, h, w, P, b.amb, b.scr1, b.bits, b.words);
  }
  if (marks)
    cudaEventRecord(marks->stage01, stream);
  const dim3 og((unsigned)order_bpf(nframes, b.words), (unsigned)nframes);
  mask_sums<<<og, kScanT, 0, stream>>>(F, b.bits, b.words, b.block_sums);
  if (K == 3) {
    // Stage 2 on the exact check's tiles, into the list positions.
    mask_prefix<<<og, kScanT, 0, stream>>>(F, b.bits, b.words, b.block_sums, b.amb, b.counters);
    const cudaError_t e = launch_lattice_stage2(F, nframes, h, w, vec, 4, P, b, stream);
    if (e != cudaSuccess)
      return e;
  } else {
    mask_list<<<og, kScanT, 0, stream>>>(b.bits, b.words, w, b.block_sums, b.cand, b.cand_cap,
                                         b.counters);
    const unsigned s2x = (unsigned)std::max(1, (8 * sms + nframes - 1) / nframes);
    seg_stage2<K><<<dim3(s2x, nframes), 256, 0, stream>>>(F, h, w, vec, P, b.scr1, b.bits,
                                                          b.words, b.cand, b.cand_cap, b.counters,
                                                          b.res);
  }
  if (marks)
    cudaEventRecord(marks->stage2, stream);
  pass_sums<<<og, kScanT, 0, stream>>>(F, b.res, b.cand_cap, b.counters, b.block_sums, b.cand,
                                       K == 3 ? b.bits : nullptr, b.words);
  pass_scatter<uint32_t><<<og, kScanT, 0, stream>>>(F, b.cand, b.cand_cap, b.res, b.counters,
                                                    b.block_sums, b.out, b.out_stride, b.capacity,
                                                    b.count_out);
  if (b.prefix) {
    mask_sums<<<og, kScanT, 0, stream>>>(F, b.bits, b.words, b.block_sums);
    mask_prefix<<<og, kScanT, 0, stream>>>(F, b.bits, b.words, b.block_sums, b.prefix, nullptr);
  }
  if (marks)
    cudaEventRecord(marks->order, stream);
  return cudaGetLastError();
}

cudaError_t launch_stream16(const FramePtrs &F, int nframes, int h, int w, const LaunchParams &P,
                            const StreamBuffers &b, int run_rows, cudaStream_t stream,
                            const StreamMarks *marks) {
  if (nframes < 1 || nframes > kMaxBatch || P.half != 3 || P.algorithm != SF_DISPERSION_EXTENDED)
    return cudaErrorInvalidValue;
  for (int f = 0; f < nframes; f++)
    if (F.w[f] % 4 != 0)
      return cudaErrorInvalidValue;
  if (marks)
    cudaEventRecord(marks->start, stream);
  cudaError_t e =
      cudaMemsetAsync(b.counters, 0, counter_words(nframes) * sizeof(uint32_t), stream);
  if (e != cudaSuccess)
    return e;
  StreamTables T;
  make_stream_tables(P, &T);
  if ((e = launch_lattice(F, nframes, h, w, 1, 2, P, T, b, run_rows, stream)) != cudaSuccess)
    return e;
  if (marks)
    cudaEventRecord(marks->stage01, stream);
  const dim3 og((unsigned)order_bpf(nframes, b.words), (unsigned)nframes);
  mask_sums<<<og, kScanT, 0, stream>>>(F, b.bits, b.words, b.block_sums);
  mask_prefix<<<og, kScanT, 0, stream>>>(F, b.bits, b.words, b.block_sums, b.amb, b.counters);
  if ((e = launch_lattice_stage2(F, nframes, h, w, 1, 2, P, b, stream)) != cudaSuccess)
    return e;
  if (marks)
    cudaEventRecord(marks->stage2, stream);
  pass_sums<<<og, kScanT, 0, stream>>>(F, b.res, b.cand_cap, b.counters, b.block_sums, b.cand,
                                       b.bits, b.words);
  pass_scatter<uint16_t><<<og, kScanT, 0, stream>>>(F, b.cand, b.cand_cap, b.res, b.counters,
                                                    b.block_sums, b.out, b.out_stride, b.capacity,
                                                    b.count_out);
  if (b.prefix) {
    mask_sums<<<og, kScanT, 0, stream>>>(F, b.bits, b.words, b.block_sums);
    mask_prefix<<<og, kScanT, 0, stream>>>(F, b.bits, b.words, b.block_sums, b.prefix, nullptr);
  }
  if (marks)
    cudaEventRecord(marks->order, stream);
  return cudaGetLastError();
}

int stream_default_run_rows(const LaunchParams &P, int h, int w, int nframes) {
  if (P.half == 3)
    return lattice_geometry(h, w, nframes, 0).run_rows;
  const int slots = P.half == 2 ? seg_slots<2>() : seg_slots<4>();
  return seg_geometry(h, w, nframes, 0, slots).run_rows;
}

cudaError_t launch_stream(const FramePtrs &F, int nframes, int h, int w, const LaunchParams &P,
                          const StreamBuffers &b, int run_rows, cudaStream_t stream,
                          const StreamMarks *marks) {
  if (nframes < 1 || nframes > kMaxBatch)
    return cudaErrorInvalidValue;
  if (marks)
    cudaEventRecord(marks->start, stream);
  cudaError_t e =
      cudaMemsetAsync(b.counters, 0, counter_words(nframes) * sizeof(uint32_t), stream);
  if (e != cudaSuccess)
    return e;
  switch (P.half) {
  case 2:
    return launch_stream_k<2>(F, nframes, h, w, P, b, run_rows, stream, marks);
  case 3:
    return launch_stream_k<3>(F, nframes, h, w, P, b, run_rows, stream, marks);
  case 4:
    return launch_stream_k<4>(F, nframes, h, w, P, b, run_rows, stream, marks);
  default:
    return cudaErrorInvalidValue;
  }
}

} // namespace sf
