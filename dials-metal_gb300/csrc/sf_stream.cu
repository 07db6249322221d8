// The streaming threshold for 32-bit frames (the benchmark path).
//
// Stage 0 and the erosion of src/spots/dext.cc (:53-142) run in one pass in
// which every warp walks down its own strip of rows; stage 2 (:151-222) runs
// afterwards only at the candidates the erosion leaves, a percent or so of
// the frame:
//
//   seg_stage01   stage 0 + erosion, one warp per 240-column strip and run
//                 of rows, no block barriers (described below)
//   stream_wide   the same outputs with 64-bit sums, for the rare runs that
//                 hold a valid pixel too large for the exact 32-bit sums
//   seg_stage2    the background-only Poisson test at each candidate, exact
//   order_*       a look-back scan of the final mask's popcounts, then every
//                 staged record scattered to its ascending position

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include <cooperative_groups.h>

#include "sf_common.cuh"
#include "sf_scan.cuh"
#include "sf_stream.cuh"

namespace cg = cooperative_groups;

namespace sf {

// Packed exact sums: the window count in the top bits (enough for the
// largest window, (2K+1)^2 pixels), the sum in the rest.
constexpr int pack_shift(int K) {
  return (2 * K + 1) * (2 * K + 1) < 32 ? 27 : (2 * K + 1) * (2 * K + 1) < 64 ? 26 : 25;
}

// ---------------------------------------------------------------------------
// Stage 0 and the erosion, one warp per (strip, run of rows).
//
// Lane l owns the 8 columns [X + 8 l, X + 8 l + 8) and walks down the run one
// pixel row at a time with no block barrier: it loads the 16 pixels
// [X + 8 l - 4, X + 8 l + 12) of the row (four 16-byte loads, the next row's
// prefetched), packs them (count and sum as n << PS | S, exact; p^2 exact in
// 32 bits), takes its 8 row sums of 2K+1 columns in registers, and carries
// 8 column sums down in registers; the row sum leaving the window comes back
// from a small per-lane ring in shared memory. Each new stage-0 row gives 8
// decisions (sf_stream.cuh), kept as 8-bit chunks in a 64-bit history; the
// erosion ANDs 2E+1 chunks vertically, then across columns with the
// neighbouring lanes' chunks (two shuffles). Lanes 0 and 31 are halo: they
// feed their neighbours' erosion and write nothing, so a warp writes 240
// columns. Pixels in the narrow range can take the near-threshold case exactly
// inline, from the exact sums, since it is rare.
// ---------------------------------------------------------------------------

constexpr int kSegLanes = 32;
constexpr int kSegOut = 240;          // output columns per warp
constexpr int kSegWarps = 4;          // warps per block
constexpr int kSegCand = 512;         // per-warp candidate buffer

template <int K> struct SegG {
  static constexpr int E = K - 1;
  static constexpr int R1 = 2 * K - 1;
  static constexpr int W0 = 2 * K + 1;
  static constexpr int N0 = W0 * W0;
  static constexpr uint32_t PS = pack_shift(K);
  static constexpr uint32_t MASK = (1u << PS) - 1u;
  static_assert(R1 <= 7, "eight rows of history");
};

template <int K> struct SegSmem {
  using G = SegG<K>;
  // ring[warp][slot][quad][lane] : uint4 = 4 of the 16 row sums
  uint4 ring[kSegWarps][G::W0][4][kSegLanes];
  uint32_t cand[kSegWarps][kSegCand];
  uint32_t ncand[kSegWarps];
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

template <int K>
__device__ void seg_flush(SegSmem<K> &s, int warp, uint32_t *cand, uint32_t *counters,
                          uint32_t cand_cap) {
  __syncwarp();
  const uint32_t n = s.ncand[warp];
  uint32_t base = 0;
  if ((threadIdx.x & 31) == 0)
    base = n ? atomicAdd(&counters[kCtrCand], n) : 0u;
  base = __shfl_sync(0xffffffffu, base, 0);
  for (uint32_t i = threadIdx.x & 31; i < n; i += 32)
    if (base + i < cand_cap)
      cand[base + i] = s.cand[warp][i];
  __syncwarp();
  if ((threadIdx.x & 31) == 0)
    s.ncand[warp] = 0;
  __syncwarp();
}

// The exact decision for the thin band neither float bound settles. Out of
// line: the common path neither carries nor issues it.
static __device__ __noinline__ bool seg_exact(uint32_t n, uint32_t S, uint32_t Q,
                                              const LaunchParams &P) {
  return stage0_u32(n, (unsigned long long)S, (unsigned long long)Q, P, P.root_lo, P.root_hi);
}

// Everything a lane carries from row to row.
template <int K> struct SegState {
  uint32_t vns[8], vq[8];
  unsigned long long hval, hs0;
  int slot;
};

// One pixel row p for this lane. Returns false when the warp must hand the
// rest of its run to the 64-bit path.
template <int K>
__device__ __forceinline__ bool seg_row(SegSmem<K> &s, SegState<K> &st, const uint32_t raw[16],
                                        int p, int p0, int ra, int rb, int cx, int X,
                                        int width, int bytes_per_row, bool writer,
                                        uint32_t inside8, int warp, int lane,
                                        const LaunchParams &P, const StreamTables &T,
                                        float nf_hi0, float c_lo0, float nf_lo0, float c_hi0,
                                        const uint32_t *__restrict__ image,
                                        uint8_t *__restrict__ scr1_bytes,
                                        uint8_t *__restrict__ final_bytes, uint32_t *cand,
                                        uint32_t cand_cap, uint32_t *counters,
                                        uint4 *wide_list) {
  using G = SegG<K>;
  constexpr int o = 4 - K;               // first of the 8 + 2K pixels used
  const uint32_t narrow = T.narrow_max;

  // Pack the pixels the row sums use.
  uint32_t ns[16], q[16];
  bool wide = false;
  uint32_t valid8 = 0;
#pragma unroll
  for (int i = o; i < o + 8 + 2 * K; i++) {
    const uint32_t v = raw[i];
    const bool small = v < narrow;
    wide |= !small && v < 0xFFFFFFFEu;
    ns[i] = small ? (v | (1u << G::PS)) : 0u;
    const uint32_t pv = small ? v : 0u;
    q[i] = pv * pv;
    if (i >= 4 && i < 12)
      valid8 |= (v < 0xFFFFFFFEu ? 1u : 0u) << (i - 4);
  }
  if (__any_sync(0xffffffffu, wide)) {
    if (lane == 0) {
      const uint32_t k = atomicAdd(&counters[kCtrWide], 1u);
      // Up to the end of the row's last mask word: the columns past the
      // frame are written as zeros there, as the lanes here would have.
      const int xb = max(0, X + 8), xe = min(bytes_per_row * 8, X + 8 + kSegOut);
      wide_list[k] =
          make_uint4((uint32_t)xb, (uint32_t)xe, (uint32_t)max(ra, p - G::R1), (uint32_t)rb);
    }
    return false;
  }
  st.hval = (st.hval << 8) | valid8;

  // Row sums of 2K + 1 columns for the 8 columns.
  uint32_t hn[8], hq[8];
  {
    uint32_t a = 0, b = 0;
#pragma unroll
    for (int d = 0; d < G::W0; d++) {
      a += ns[o + d];
      b += q[o + d];
    }
    hn[0] = a;
    hq[0] = b;
#pragma unroll
    for (int c = 1; c < 8; c++) {
      a += ns[o + c + 2 * K] - ns[o + c - 1];
      b += q[o + c + 2 * K] - q[o + c - 1];
      hn[c] = a;
      hq[c] = b;
    }
  }

  // Column sums: the row sums of W0 rows ago come back from the ring.
  {
    uint4 *r = &s.ring[warp][st.slot][0][lane];
    const uint4 l0 = r[0], l1 = r[32], l2 = r[64], l3 = r[96];
    const uint32_t ln[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
    const uint32_t lq[8] = {l2.x, l2.y, l2.z, l2.w, l3.x, l3.y, l3.z, l3.w};
#pragma unroll
    for (int c = 0; c < 8; c++) {
      st.vns[c] += hn[c] - ln[c];
      st.vq[c] += hq[c] - lq[c];
    }
    r[0] = make_uint4(hn[0], hn[1], hn[2], hn[3]);
    r[32] = make_uint4(hn[4], hn[5], hn[6], hn[7]);
    r[64] = make_uint4(hq[0], hq[1], hq[2], hq[3]);
    r[96] = make_uint4(hq[4], hq[5], hq[6], hq[7]);
    st.slot = st.slot + 1 == G::W0 ? 0 : st.slot + 1;
  }
  if (p < p0 + 2 * K)
    return true;  // the column sums are not yet full windows (warp-uniform)

  // Stage-0 row p - K: eight decisions.
  uint32_t s8 = 0;
  const uint32_t vrow = (uint32_t)(st.hval >> (8 * K)) & 0xFFu;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    bool bit = !((vrow >> c) & 1u);  // masked pixels are set
    if (!bit) {
      const uint32_t n = st.vns[c] >> G::PS, S = st.vns[c] & G::MASK;
      const bool full = n == (uint32_t)G::N0;
      const float Sf = __uint2float_rn(S), Qf = __uint2float_rn(st.vq[c]);
      // Surely not: nQ <= S (S + c) (bounds in sf_stream.cuh).
      if (!(__fmul_rn(full ? nf_hi0 : T.nf_hi[n], Qf) <=
            __fmul_rn(Sf, __fadd_rn(Sf, full ? c_lo0 : T.c_lo[n])))) {
        // Surely: nQ >= S (S + c) + 1; otherwise decide exactly (rare).
        if (__fmul_rn(full ? nf_lo0 : T.nf_lo[n], Qf) >=
            __fadd_rn(__fmul_rn(__fmul_rn(Sf, __fadd_rn(Sf, full ? c_hi0 : T.c_hi[n])), 1.0001f),
                      2.0f))
          bit = true;
        else
          bit = seg_exact(n, S, st.vq[c], P);
      }
    }
    s8 |= (bit ? 1u : 0u) << c;
  }
  st.hs0 = (st.hs0 << 8) | s8;
  if (p < p0 + 2 * K + 2 * G::E)
    return true;  // the erosion needs 2E more decision rows (warp-uniform)

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
  const uint32_t scr1 = (h8 | masked8) & inside8;
  const int re = p - G::R1;
  const bool out_row = re >= ra && re < rb;
  if (out_row && writer) {
    scr1_bytes[(size_t)re * bytes_per_row + (cx >> 3)] = (uint8_t)scr1;
    final_bytes[(size_t)re * bytes_per_row + (cx >> 3)] = 0;
  }
  // Candidates: eroded, not masked, above the global threshold.
  uint32_t c8 = (out_row && writer) ? (scr1 & ~masked8) : 0u;
  if (__any_sync(0xffffffffu, c8 != 0u)) {
    if (c8) {
      const uint32_t *row = image + (size_t)re * width;
#pragma unroll
      for (int c = 0; c < 8; c++)
        if (((c8 >> c) & 1u) && (uint64_t)__ldg(row + cx + c) < P.p_min)
          c8 &= ~(1u << c);
    }
    const uint32_t cnt = __popc(c8);
    uint32_t incl = cnt;
#pragma unroll
    for (int o2 = 1; o2 < 32; o2 <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o2);
      if (lane >= o2)
        incl += t;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (s.ncand[warp] + total > (uint32_t)kSegCand)
      seg_flush<K>(s, warp, cand, counters, cand_cap);
    const uint32_t base = s.ncand[warp] + incl - cnt;
    uint32_t k = 0;
    for (int c = 0; c < 8; c++)
      if ((c8 >> c) & 1u)
        s.cand[warp][base + k++] = (uint32_t)re * (uint32_t)width + (uint32_t)(cx + c);
    __syncwarp();
    if (lane == 0)
      s.ncand[warp] += total;
    __syncwarp();
  }
  return true;
}

template <int K>
__global__ void __launch_bounds__(kSegWarps * 32, 3)
seg_stage01(const uint32_t *__restrict__ image, int height, int width, int vec, int nstrips,
            int nruns, int run_rows, const __grid_constant__ LaunchParams P,
            const __grid_constant__ StreamTables T, uint8_t *__restrict__ scr1_bytes,
            uint8_t *__restrict__ final_bytes, uint32_t *__restrict__ cand, uint32_t cand_cap,
            uint32_t *__restrict__ counters, uint4 *__restrict__ wide_list) {
  using G = SegG<K>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SegSmem<K> &s = *reinterpret_cast<SegSmem<K> *>(smem_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gw = blockIdx.x * kSegWarps + warp;
  const int sx = gw % nstrips, ry = gw / nstrips;
  if (ry >= nruns)
    return;  // whole warp
  const int X = kSegOut * sx - 8;
  const int cx = X + 8 * lane;
  const int ra = ry * run_rows;
  const int rb = min(height, ra + run_rows);
  const int bytes_per_row = ((width + 31) >> 5) * 4;
  const bool writer = lane >= 1 && lane <= 30 && cx < bytes_per_row * 8;
  const bool interior = vec && cx - 4 >= 0 && cx + 12 <= width;
  const float nf_hi0 = T.nf_hi[G::N0], c_lo0 = T.c_lo[G::N0];
  const float nf_lo0 = T.nf_lo[G::N0], c_hi0 = T.c_hi[G::N0];
  // Bits of this lane's columns that lie inside the frame.
  const uint32_t inside8 =
      cx >= width ? 0u : (cx + 8 <= width ? 0xFFu : ((1u << (width - cx)) - 1u));

  if (lane == 0)
    s.ncand[warp] = 0;
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

  const int p0 = ra - G::R1, p1 = rb + G::R1;  // pixel rows [p0, p1)
  uint32_t A[16], B[16];
  seg_load(image, height, width, interior, cx, p0, A);
  for (int p = p0; p < p1; p += 2) {
    // Two rows per pass, the loads alternating between A and B.
    if (p + 1 < p1)
      seg_load(image, height, width, interior, cx, p + 1, B);
    if (!seg_row<K>(s, st, A, p, p0, ra, rb, cx, X, width, bytes_per_row, writer, inside8,
                    warp, lane, P, T, nf_hi0, c_lo0, nf_lo0, c_hi0, image, scr1_bytes,
                    final_bytes, cand, cand_cap, counters, wide_list))
      break;
    if (p + 1 >= p1)
      break;
    if (p + 2 < p1)
      seg_load(image, height, width, interior, cx, p + 2, A);
    if (!seg_row<K>(s, st, B, p + 1, p0, ra, rb, cx, X, width, bytes_per_row, writer,
                    inside8, warp, lane, P, T, nf_hi0, c_lo0, nf_lo0, c_hi0, image,
                    scr1_bytes, final_bytes, cand, cand_cap, counters, wide_list))
      break;
  }
  seg_flush<K>(s, warp, cand, counters, cand_cap);
}

// ---------------------------------------------------------------------------
// Runs holding a pixel too large for the exact 32-bit sums: 32 x 32 tiles of
// the eroded mask with 64-bit sums, for the columns [xb, xe) and rows
// [yb, ye) a warp handed over.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(256)
stream_wide(const uint32_t *__restrict__ image, int height, int width, int run_rows,
            const __grid_constant__ LaunchParams P, uint8_t *__restrict__ scr1_bytes,
            uint8_t *__restrict__ final_bytes, uint32_t *__restrict__ cand,
            uint32_t cand_cap, uint32_t *__restrict__ counters,
            const uint4 *__restrict__ wide_list) {
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
    const uint4 w = wide_list[item / (TPS * TPR)];
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
      if (gy < ty1 && lane < 4) {
        const int bx = tx0 + 8 * lane;
        if (bx < xe && (bx >> 3) < bytes_per_row) {
          scr1_bytes[(size_t)gy * bytes_per_row + (bx >> 3)] = (uint8_t)(word >> (8 * lane));
          final_bytes[(size_t)gy * bytes_per_row + (bx >> 3)] = 0;
        }
      }
      const bool cnd = b && v < 0xFFFFFFFEu && (uint64_t)v >= P.p_min;
      const unsigned cm = __ballot_sync(0xffffffffu, cnd);
      if (cm) {
        uint32_t base = 0;
        if (lane == 0)
          base = atomicAdd(&counters[kCtrCand], (uint32_t)__popc(cm));
        base = __shfl_sync(0xffffffffu, base, 0);
        const uint32_t g = base + __popc(cm & ((1u << lane) - 1u));
        if (cnd && g < cand_cap)
          cand[g] = (uint32_t)gy * (uint32_t)width + (uint32_t)gx;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Stage 2 at the candidates, four lanes to a candidate: each lane sums a
// quarter of the (2K + 5) rows of the clipped window, two shuffles add them.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(256)
seg_stage2(const uint32_t *__restrict__ image, int height, int width,
           const __grid_constant__ LaunchParams P, const uint32_t *__restrict__ scr1_words,
           uint32_t *__restrict__ final_words, const uint32_t *__restrict__ cand,
           uint32_t cand_cap, uint32_t *__restrict__ counters,
           sf_signal_pixel *__restrict__ staging, uint32_t capacity) {
  constexpr int K2 = K + 2, WW = 2 * K2 + 1;
  const int wpr = (width + 31) >> 5;
  const uint32_t nc = min(counters[kCtrCand], cand_cap);
  const int lane = threadIdx.x & 31, sub = lane & 3;
  const uint32_t per_pass = (gridDim.x * blockDim.x) >> 2;
  for (uint32_t base = (blockIdx.x * blockDim.x) >> 2; base < nc + 0; base += per_pass) {
    const uint32_t i = base + (threadIdx.x >> 2);
    const bool live = i < nc;
    uint32_t idx = 0, p = 0, n = 0;
    unsigned long long S = 0;
    if (live) {
      idx = cand[i];
      const int y = (int)(idx / (uint32_t)width), x = (int)(idx % (uint32_t)width);
      p = __ldg(image + idx);
      const int xlo = max(0, x - K2), xhi = min(width - 1, x + K2);
      const int w0 = xlo >> 5;
      constexpr int ROWS = (WW + 3) / 4;  // rows per lane
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
        uint32_t v[WW];
#pragma unroll
        for (int d = 0; d < WW; d++)
          v[d] = (xlo + d <= xhi) ? __ldg(row + xlo + d) : 0u;
#pragma unroll
        for (int d = 0; d < WW; d++)
          if (xlo + d <= xhi && ((bgb >> d) & 1ull)) {
            // Not in the eroded mask, so valid (masked pixels are in it).
            n++;
            S += v[d];
          }
      }
    }
    n += __shfl_xor_sync(0xffffffffu, n, 1);
    S += __shfl_xor_sync(0xffffffffu, S, 1);
    n += __shfl_xor_sync(0xffffffffu, n, 2);
    S += __shfl_xor_sync(0xffffffffu, S, 2);
    bool sig = false;
    sf_signal_pixel rec;
    if (live && sub == 0) {
      float bg;
      sig = stage2_u32(p, n, S, P, &bg);
      rec.index = idx;
      rec.value = p;
      rec.background = bg;
      rec.population = (uint16_t)n;
      rec.reserved = 0;
    }
    const unsigned m = __ballot_sync(0xffffffffu, sig);
    if (m) {
      uint32_t b = 0;
      if (lane == 0)
        b = atomicAdd(&counters[kCtrTotal], (uint32_t)__popc(m));
      b = __shfl_sync(0xffffffffu, b, 0);
      if (sig) {
        const uint32_t slot = b + __popc(m & ((1u << lane) - 1u));
        if (slot < capacity)
          staging[slot] = rec;
        const uint32_t y = idx / (uint32_t)width, x = idx % (uint32_t)width;
        atomicOr(&final_words[(size_t)y * wpr + (x >> 5)], 1u << (x & 31u));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Ordering, one cooperative kernel with one block per SM: each block sums
// the popcounts of its share of the final mask's words; after a grid-wide
// barrier each block adds its predecessors' sums and writes the exclusive
// prefix of every word it owns; after a second barrier every staged record is
// scattered to its ascending position.
// ---------------------------------------------------------------------------
constexpr int kOrderThreads = 1024;

__global__ void __launch_bounds__(kOrderThreads)
order_coop(int width, const uint32_t *__restrict__ bits, uint32_t nwords,
           uint32_t *__restrict__ prefix, uint32_t *__restrict__ block_sums,
           const uint32_t *__restrict__ counters, uint32_t cand_cap,
           const sf_signal_pixel *__restrict__ staging, uint32_t capacity,
           sf_signal_pixel *__restrict__ out, uint32_t *__restrict__ count_out) {
  cg::grid_group grid = cg::this_grid();
  const uint32_t chunk = (nwords + gridDim.x - 1) / gridDim.x;
  const uint32_t lo = min(nwords, blockIdx.x * chunk), hi = min(nwords, lo + chunk);
  uint32_t acc = 0;
  for (uint32_t w = lo + threadIdx.x; w < hi; w += blockDim.x)
    acc += __popc(bits[w]);
  uint32_t total;
  (void)block_exclusive_scan(acc, &total);
  if (threadIdx.x == 0)
    block_sums[blockIdx.x] = total;
  grid.sync();
  __shared__ uint32_t s_base;
  if (threadIdx.x < 32) {
    uint32_t b = 0;
    for (uint32_t i = threadIdx.x; i < blockIdx.x; i += 32)
      b += block_sums[i];
    for (int o = 16; o; o >>= 1)
      b += __shfl_xor_sync(0xffffffffu, b, o);
    if (threadIdx.x == 0)
      s_base = b;
  }
  __syncthreads();
  uint32_t carry = s_base;
  for (uint32_t base = lo; base < hi; base += blockDim.x) {
    const uint32_t w = base + threadIdx.x;
    const uint32_t c = w < hi ? __popc(bits[w]) : 0u;
    uint32_t t;
    const uint32_t e = block_exclusive_scan(c, &t);
    if (w < hi)
      prefix[w] = carry + e;
    carry += t;
  }
  grid.sync();
  const uint32_t found = counters[kCtrTotal];
  if (blockIdx.x == 0 && threadIdx.x == 0)
    // The signal found; all ones if the candidate list overflowed, as for a
    // count above capacity (the list is then incomplete).
    *count_out = counters[kCtrCand] > cand_cap ? 0xFFFFFFFFu : found;
  const uint32_t n = min(found, capacity);
  const int wpr = (width + 31) >> 5;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const sf_signal_pixel rec = staging[i];
    const uint32_t y = rec.index / (uint32_t)width, x = rec.index % (uint32_t)width;
    const size_t w = (size_t)y * wpr + (x >> 5);
    const uint32_t dst = prefix[w] + __popc(bits[w] & ((1u << (x & 31u)) - 1u));
    if (dst < capacity)
      out[dst] = rec;
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------

static float round_down(double v) {
  float f = (float)v;
  if ((double)f > v)
    f = nextafterf(f, -INFINITY);
  return f;
}
static float round_up(double v) {
  float f = (float)v;
  if ((double)f < v)
    f = nextafterf(f, INFINITY);
  return f;
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
    // c = n - 1 + sigma_b r_n with the reference's double r_n; the margins
    // are 2^-14 relative on n, far above the ~2^-19 the float sums can err.
    // The double sum itself may round, hence the 2^-40 widening.
    const double c = testable ? (double)(n - 1) + (double)P.sigma_b_int * P.root[n] : 0.0;
    T->c_lo[n] = testable ? round_down(c * (1.0 - 0x1p-40)) : 0.0f;
    T->c_hi[n] = testable ? round_up(c * (1.0 + 0x1p-40)) : 0.0f;
    T->nf_hi[n] = testable ? round_up((double)n * (1.0 + 1.0 / 16384.0)) : 0.0f;
    // Untestable windows are never signal: nf_lo 0 keeps "surely" false.
    T->nf_lo[n] = testable ? round_down((double)n * (1.0 - 1.0 / 16384.0)) : 0.0f;
  }
}

// One block per SM for the cooperative ordering kernel.
static int order_blocks() {
  static int n = 0;
  if (!n) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, order_coop, kOrderThreads, 0);
    n = sms * (per > 0 ? 1 : 0);
    if (n <= 0)
      n = 1;
    if (n > kScanBlocks)
      n = kScanBlocks;
  }
  return n;
}

template <int K>
static cudaError_t launch_stream_k(const uint32_t *image, int h, int w, const LaunchParams &P,
                                   const StreamBuffers &b, cudaStream_t stream) {
  using S = SegSmem<K>;
  static bool configured = false;
  cudaError_t e;
  if (!configured) {
    e = cudaFuncSetAttribute(seg_stage01<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(S));
    if (e != cudaSuccess)
      return e;
    configured = true;
  }
  StreamTables T;
  make_stream_tables(P, &T);
  const int vec = (w % 4 == 0 && reinterpret_cast<uintptr_t>(image) % 16 == 0) ? 1 : 0;
  const SegGeometry g = seg_geometry(h, w);
  const int warps = g.nstrips * g.nruns;
  uint8_t *scr1 = reinterpret_cast<uint8_t *>(b.scr1);
  uint8_t *fin = reinterpret_cast<uint8_t *>(b.bits);
  seg_stage01<K><<<(warps + kSegWarps - 1) / kSegWarps, kSegWarps * 32, sizeof(S), stream>>>(
      image, h, w, vec, g.nstrips, g.nruns, g.run_rows, P, T, scr1, fin, b.cand, b.cand_cap,
      b.counters, b.wide);
  stream_wide<K><<<2 * 152, 256, 0, stream>>>(image, h, w, g.run_rows, P, scr1, fin, b.cand,
                                               b.cand_cap, b.counters, b.wide);
  seg_stage2<K><<<8 * 152, 256, 0, stream>>>(image, h, w, P, b.scr1, b.bits, b.cand,
                                              b.cand_cap, b.counters, b.staging, b.capacity);
  uint32_t nwords = (uint32_t)(((size_t)w + 31) / 32 * h);
  int width = w;
  uint32_t cand_cap = b.cand_cap, capacity = b.capacity;
  const uint32_t *bits_c = b.bits;
  const uint32_t *counters_c = b.counters;
  const sf_signal_pixel *staging_c = b.staging;
  void *args[] = {&width,    &bits_c,    &nwords,    (void *)&b.prefix, (void *)&b.block_sums,
                  &counters_c, &cand_cap, &staging_c, &capacity,         (void *)&b.out,
                  (void *)&b.count_out};
  e = cudaLaunchCooperativeKernel((void *)order_coop, dim3(order_blocks()), dim3(kOrderThreads),
                                  args, 0, stream);
  if (e != cudaSuccess)
    return e;
  return cudaGetLastError();
}

cudaError_t launch_stream(const uint32_t *image, int h, int w, const LaunchParams &P,
                          const StreamBuffers &b, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(b.counters, 0, kCtrCount * sizeof(uint32_t), stream);
  if (e != cudaSuccess)
    return e;
  switch (P.half) {
  case 2:
    return launch_stream_k<2>(image, h, w, P, b, stream);
  case 3:
    return launch_stream_k<3>(image, h, w, P, b, stream);
  case 4:
    return launch_stream_k<4>(image, h, w, P, b, stream);
  default:
    return cudaErrorInvalidValue;
  }
}

} // namespace sf
