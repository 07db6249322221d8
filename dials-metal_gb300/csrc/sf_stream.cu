// The streaming threshold for 32-bit frames (the benchmark path).
//
// Stage 0 and the erosion of src/spots/dext.cc (:53-142) run in one pass
// down vertical strips; stage 2 (:151-222) runs afterwards only at the
// candidates the erosion leaves, which are a percent or so of the frame.
//
//   stream_stage01   One block per strip segment: 224 output columns by 96
//                    output rows, walking down in steps of 8 rows. Each step
//                    packs 8 new pixel rows into shared memory (count and sum
//                    as n << 26 | S, exact; I^2 as float), takes row sums of
//                    2K+1 columns, then one thread per column carries the
//                    column sums down in registers and decides the dispersion
//                    test for its pixel with a float bound: "surely not",
//                    "surely", or near the threshold, in which case the pixel
//                    is queued and decided exactly (uint64 sums, then the
//                    reference's integer/double decision, sf_common.cuh). The
//                    stage-0 mask lives in per-column shift registers, so the
//                    erosion is a few shifts and ANDs. Out: the eroded mask
//                    (bitmask), the final mask zeroed, and the candidates.
//   stream_wide      The same outputs with 64-bit sums, for the rare strip
//                    segments holding a valid pixel too large for the packed
//                    sums (>= 2^26 / n_max); stream_stage01 hands them over
//                    from the row where it met one.
//   stream_stage2    One thread per candidate: the background count and sum
//                    over the clipped (2K+5)^2 window, the Poisson test
//                    (exact, sf_common.cuh), the record into a staging list and
//                    the bit into the final mask.
//   order_*          Popcount prefix of the final mask's words, then every
//                    staged record scattered to its ascending position.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "sf_common.cuh"
#include "sf_scan.cuh"
#include "sf_stream.cuh"

namespace sf {

// Packed exact sums: the window count in the top bits (enough for the
// largest window, (2K+1)^2 pixels), the sum in the rest.
constexpr int pack_shift(int K) {
  return (2 * K + 1) * (2 * K + 1) < 32 ? 27 : (2 * K + 1) * (2 * K + 1) < 64 ? 26 : 25;
}

template <int K> struct SG {
  static constexpr int E = K - 1;          // erosion radius
  static constexpr int R1 = 2 * K - 1;     // pixel halo of the eroded mask
  static constexpr int A = 8;              // left pad: >= R1, 16-byte aligned
  static constexpr int TW = kStreamTW;     // output columns per strip (224)
  static constexpr int LW = TW + 2 * A;    // loaded columns (240)
  static constexpr int LWP = LW + 8;       // ring row stride (reads run past LW)
  static constexpr int S0W = TW + 2 * E;   // stage-0 columns
  static constexpr int NT = 256;
  static constexpr int STEP = 8;
  static constexpr int RING = 16;          // packed-pixel ring rows
  static constexpr int NSEG = (S0W + 7) / 8;
  static constexpr int HW = NSEG * 8;      // row-sum stride
  static constexpr int NWORD = TW / 32;
  static constexpr int N0 = (2 * K + 1) * (2 * K + 1);
  static constexpr int F4 = LW / 4;        // float4 per loaded row
  static constexpr int CCAP = 2048;        // block candidate buffer
  static constexpr uint32_t PS = pack_shift(K);
  static constexpr uint32_t MASK = (1u << PS) - 1u;
  static_assert(N0 < (1 << (32 - PS)), "the count fits above the sum");
  static_assert(TW % 32 == 0, "strip width is whole words");
  static_assert(S0W <= NT, "one thread per stage-0 column");
  static_assert(A >= R1 && A % 4 == 0, "pad");
  static_assert(8 * (NSEG - 1) + 19 < LWP, "row-sum reads stay in the row");
  static_assert(A - R1 + 7 + 2 * K <= 19, "a segment's windows lie in its 20 loaded values");
};


__device__ __forceinline__ float u23_to_float(uint32_t v) {
  // Exact for v < 2^23: the bits of 2^23 + v, less 2^23.
  return __fsub_rn(__uint_as_float(v | 0x4B000000u), 8388608.0f);
}

template <int K>
struct StreamSmem {
  using G = SG<K>;
  uint32_t ns[G::RING][G::LWP];      // packed pixels: valid ? (1 << PS | p) : 0
  uint32_t q[G::STEP][G::LWP];       // p^2, the step's rows
  uint32_t hns[G::STEP][G::HW];      // row sums of packed pixels
  uint32_t hq[G::STEP][G::HW];       // row sums of p^2
  uint32_t vcol[G::S0W];             // vertical erosion words
  uint32_t fix[G::S0W];              // exact decisions that came out "signal"
  uint16_t defer[G::S0W * G::STEP];  // queued pixels: j * 8 + row-in-step
  uint32_t cand[G::CCAP];
  float nf_hi[G::N0 + 1], nf_lo[G::N0 + 1], c_lo[G::N0 + 1], c_hi[G::N0 + 1];
  uint32_t root_lo[G::N0 + 1], root_hi[G::N0 + 1];
  uint32_t ndefer, ncand;
};

template <int K>
__device__ void flush_candidates(StreamSmem<K> &s, uint32_t *cand, uint32_t *counters,
                                 uint32_t cand_cap) {
  // All threads; s.ncand stable (called between barriers).
  const uint32_t n = s.ncand;
  __shared__ uint32_t base;
  if (threadIdx.x == 0)
    base = n ? atomicAdd(&counters[kCtrCand], n) : 0u;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    const uint32_t g = base + i;
    if (g < cand_cap)
      cand[g] = s.cand[i];
  }
  __syncthreads();
  if (threadIdx.x == 0)
    s.ncand = 0;
  __syncthreads();
}

// One step's raw pixels for this thread: float4 number tid and tid + 256 of
// the step's 8 x F4.
template <int K>
__device__ __forceinline__ void load_step(const uint32_t *__restrict__ image, int height,
                                          int width, int vec, int x0, int P0, uint4 v[2]) {
  using G = SG<K>;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int i = threadIdx.x + h * G::NT;
    v[h] = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
    if (i >= G::STEP * G::F4)
      continue;
    const int r = i / G::F4, c4 = i - r * G::F4;
    const int gy = P0 + r, gx = x0 - G::A + 4 * c4;
    if (gy < 0 || gy >= height)
      continue;
    const uint32_t *row = image + (size_t)gy * width;
    if (vec && gx >= 0 && gx + 3 < width) {
      v[h] = __ldg(reinterpret_cast<const uint4 *>(row + gx));
    } else {
      uint32_t t[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
#pragma unroll
      for (int e = 0; e < 4; e++)
        if (gx + e >= 0 && gx + e < width)
          t[e] = __ldg(row + gx + e);
      v[h] = make_uint4(t[0], t[1], t[2], t[3]);
    }
  }
}

template <int K>
__global__ void __launch_bounds__(256, 3)
stream_stage01(const uint32_t *__restrict__ image, int height, int width, int vec,
               const __grid_constant__ LaunchParams P, const __grid_constant__ StreamTables T,
               uint32_t *__restrict__ scr1_bits, uint32_t *__restrict__ final_bits,
               uint32_t *__restrict__ cand, uint32_t cand_cap, uint32_t *__restrict__ counters,
               uint4 *__restrict__ wide_list) {
  using G = SG<K>;
  constexpr int W0 = 2 * K + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  StreamSmem<K> &s = *reinterpret_cast<StreamSmem<K> *>(smem_raw);
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int x0 = blockIdx.x * G::TW;
  const int y0 = blockIdx.y * kStreamSH;
  const int y1 = min(height, y0 + kStreamSH);
  const int wpr = (width + 31) >> 5;
  const uint32_t narrow = T.narrow_max;
  // The all-valid window's table entries, the common case.
  const float nf_hi0 = T.nf_hi[G::N0], nf_lo0 = T.nf_lo[G::N0];
  const float c_lo0 = T.c_lo[G::N0], c_hi0 = T.c_hi[G::N0];

  for (int i = tid; i <= G::N0; i += G::NT) {
    s.nf_hi[i] = T.nf_hi[i];
    s.nf_lo[i] = T.nf_lo[i];
    s.c_lo[i] = T.c_lo[i];
    s.c_hi[i] = T.c_hi[i];
    s.root_lo[i] = P.root_lo[i];
    s.root_hi[i] = P.root_hi[i];
  }
  for (int i = tid; i < G::RING * G::LWP; i += G::NT)
    (&s.ns[0][0])[i] = 0u;
  for (int i = tid; i < G::S0W; i += G::NT)
    s.fix[i] = 0u;
  if (tid == 0) {
    s.ndefer = 0;
    s.ncand = 0;
  }

  // This thread's stage-0 column j (output column j - E), if any.
  int j = -1;
  if (tid < G::TW)
    j = tid + G::E;
  else if (tid < G::TW + G::E)
    j = tid - G::TW;
  else if (tid < G::TW + 2 * G::E)
    j = tid;
  const bool own = j >= 0;
  const int cj = G::A - G::E + (own ? j : 0);  // its column in the loaded rows

  // Row sums of the previous two steps (index i = row P0 - 8 + i for old,
  // P0 - 16 + i for old2).
  uint32_t old_ns[8], old2_ns[8], old_q[8], old2_q[8];
#pragma unroll
  for (int i = 0; i < 8; i++)
    old_ns[i] = old2_ns[i] = old_q[i] = old2_q[i] = 0u;
  uint32_t vns = 0, vq = 0; // running column sums
  uint32_t sreg = 0;        // stage-0 mask, bit 0 = newest row
  uint32_t mreg = 0;        // masked pixels, same rows

  const int p_first = y0 - G::R1;
  uint4 raw[2];
  load_step<K>(image, height, width, vec, x0, p_first, raw);
  __syncthreads();

  // Ring rows are indexed by row - p_first (non-negative) modulo RING.
  for (int P0 = p_first;; P0 += G::STEP) {
    const int newest_v0 = P0 + 7 - K;
    const int out_hi = newest_v0 - G::E;  // highest eroded row this step
    const int out_lo = out_hi - 7;
    if (out_lo >= y1)
      break;
    const int rb = P0 - p_first;          // ring base for row P0

    // -- pack the step's 8 pixel rows; prefetch the next step's ---------------
    bool wide = false;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int i = tid + h * G::NT;
      if (i < G::STEP * G::F4) {
        const int r = i / G::F4, c4 = i - r * G::F4;
        const uint32_t v[4] = {raw[h].x, raw[h].y, raw[h].z, raw[h].w};
        uint32_t pk[4], qq[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const bool valid = v[e] < 0xFFFFFFFEu;
          wide |= valid && v[e] >= narrow;
          const uint32_t pv = valid && v[e] < narrow ? v[e] : 0u;
          pk[e] = valid ? ((1u << G::PS) | pv) : 0u;
          qq[e] = pv * pv;
        }
        *reinterpret_cast<uint4 *>(&s.ns[(rb + r) & (G::RING - 1)][4 * c4]) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
        *reinterpret_cast<uint4 *>(&s.q[r][4 * c4]) = make_uint4(qq[0], qq[1], qq[2], qq[3]);
      }
    }
    load_step<K>(image, height, width, vec, x0, P0 + G::STEP, raw);
    if (__syncthreads_or(wide)) {
      // Rows from out_lo on are not yet written: hand the rest over.
      if (tid == 0) {
        const uint32_t k = atomicAdd(&counters[kCtrWide], 1u);
        wide_list[k] = make_uint4((uint32_t)x0, (uint32_t)max(out_lo, y0), (uint32_t)y1, 0u);
      }
      break;
    }

    // -- row sums over 2K + 1 columns, 8 outputs per thread ------------------
    if (tid < G::STEP * G::NSEG) {
      const int r = tid / G::NSEG, sg = tid - r * G::NSEG;
      const int ring_r = (rb + r) & (G::RING - 1);
      const int c0 = 8 * sg;
      uint32_t a[20], b[20];
#pragma unroll
      for (int f = 0; f < 5; f++) {
        const uint4 u = *reinterpret_cast<const uint4 *>(&s.ns[ring_r][c0 + 4 * f]);
        const uint4 w = *reinterpret_cast<const uint4 *>(&s.q[r][c0 + 4 * f]);
        a[4 * f] = u.x, a[4 * f + 1] = u.y, a[4 * f + 2] = u.z, a[4 * f + 3] = u.w;
        b[4 * f] = w.x, b[4 * f + 1] = w.y, b[4 * f + 2] = w.z, b[4 * f + 3] = w.w;
      }
      constexpr int o = G::A - G::R1;
      uint32_t hn[8], hq[8];
      uint32_t ra = 0, rq = 0;
#pragma unroll
      for (int d = 0; d < W0; d++) {
        ra += a[o + d];
        rq += b[o + d];
      }
      hn[0] = ra;
      hq[0] = rq;
#pragma unroll
      for (int k = 1; k < 8; k++) {
        ra += a[o + k + 2 * K] - a[o + k - 1];
        rq += b[o + k + 2 * K] - b[o + k - 1];
        hn[k] = ra;
        hq[k] = rq;
      }
      *reinterpret_cast<uint4 *>(&s.hns[r][c0]) = make_uint4(hn[0], hn[1], hn[2], hn[3]);
      *reinterpret_cast<uint4 *>(&s.hns[r][c0 + 4]) = make_uint4(hn[4], hn[5], hn[6], hn[7]);
      *reinterpret_cast<uint4 *>(&s.hq[r][c0]) = make_uint4(hq[0], hq[1], hq[2], hq[3]);
      *reinterpret_cast<uint4 *>(&s.hq[r][c0 + 4]) = make_uint4(hq[4], hq[5], hq[6], hq[7]);
    }
    __syncthreads();

    // -- column sums and the dispersion test, one thread per column ----------
    {
      uint32_t cur_ns[8], cur_q[8];
#pragma unroll
      for (int r = 0; r < 8; r++) {
        cur_ns[r] = own ? s.hns[r][j] : 0u;
        cur_q[r] = own ? s.hq[r][j] : 0u;
      }
#pragma unroll
      for (int r = 0; r < 8; r++) {
        // The row sums leaving the 2K + 1 window (static indices).
        constexpr int dummy = 0;
        (void)dummy;
        const int d = r - W0;
        const uint32_t lns = d >= 0 ? cur_ns[d >= 0 ? d : 0]
                             : d >= -8 ? old_ns[d >= -8 ? 8 + d : 0]
                                       : old2_ns[16 + d >= 0 ? 16 + d : 0];
        const uint32_t lq = d >= 0 ? cur_q[d >= 0 ? d : 0]
                            : d >= -8 ? old_q[d >= -8 ? 8 + d : 0]
                                      : old2_q[16 + d >= 0 ? 16 + d : 0];
        vns += cur_ns[r] - lns;
        vq += cur_q[r] - lq;
        // Stage-0 row P0 + r - K.
        const uint32_t me = s.ns[(rb + r - K + G::RING) & (G::RING - 1)][cj];
        const bool masked = me == 0u;
        bool bit = masked, defer = false;
        if (!masked) {
          const uint32_t n = vns >> G::PS;
          const uint32_t S = vns & G::MASK;
          const bool full = n == (uint32_t)G::N0;
          const float nhi = full ? nf_hi0 : s.nf_hi[n];
          const float clo = full ? c_lo0 : s.c_lo[n];
          const float Sf = __uint2float_rn(S);
          const float Qf = __uint2float_rn(vq);
          // Surely not: nQ <= S (S + c) (bounds in sf_stream.cuh).
          if (!(__fmul_rn(nhi, Qf) <= __fmul_rn(Sf, __fadd_rn(Sf, clo)))) {
            const float nlo = full ? nf_lo0 : s.nf_lo[n];
            const float chi = full ? c_hi0 : s.c_hi[n];
            // Surely: nQ >= S (S + c) + 1.
            if (__fmul_rn(nlo, Qf) >=
                __fadd_rn(__fmul_rn(__fmul_rn(Sf, __fadd_rn(Sf, chi)), 1.0001f), 2.0f))
              bit = true;
            else {
              const int row = P0 + r - K;
              // Rows beyond these only feed outputs outside the segment.
              defer = own && row >= y0 - G::E && row < y1 + G::E;
            }
          }
        }
        if (__any_sync(0xffffffffu, defer)) {
          const unsigned dm = __ballot_sync(0xffffffffu, defer);
          uint32_t base = 0;
          if (lane == 0)
            base = atomicAdd(&s.ndefer, (uint32_t)__popc(dm));
          base = __shfl_sync(0xffffffffu, base, 0);
          if (defer)
            s.defer[base + __popc(dm & ((1u << lane) - 1u))] = (uint16_t)(j * 8 + r);
        }
        sreg = (sreg << 1) | (bit ? 1u : 0u);
        mreg = (mreg << 1) | (masked ? 1u : 0u);
      }
#pragma unroll
      for (int r = 0; r < 8; r++) {
        old2_ns[r] = old_ns[r];
        old_ns[r] = cur_ns[r];
        old2_q[r] = old_q[r];
        old_q[r] = cur_q[r];
      }
    }
    __syncthreads();

    // -- the queued pixels, decided exactly (rare) ----------------------------
    {
      const uint32_t nd = s.ndefer;
      for (uint32_t i = tid; i < nd; i += G::NT) {
        const uint32_t e = s.defer[i];
        const int jj = (int)(e >> 3), r = (int)(e & 7u);
        const int c = G::A - G::E + jj;
        uint32_t n = 0;
        unsigned long long S = 0, Q = 0;
        for (int dy = -K; dy <= K; dy++) {
          const int ring_r = (rb + r - K + dy + G::RING) & (G::RING - 1);
          for (int dx = -K; dx <= K; dx++) {
            const uint32_t v = s.ns[ring_r][c + dx];
            if (v) {
              const unsigned long long p = v & G::MASK;
              n++;
              S += p;
              Q += p * p;
            }
          }
        }
        if (stage0_u32(n, S, Q, P, s.root_lo, s.root_hi))
          atomicOr(&s.fix[jj], 1u << (7 - r));
      }
    }
    __syncthreads();
    if (tid == 0)
      s.ndefer = 0;

    // -- erosion ---------------------------------------------------------------
    if (own) {
      sreg |= s.fix[j];
      s.fix[j] = 0u;
      uint32_t v = sreg;
#pragma unroll
      for (int d = 1; d <= G::E; d++)
        v &= (sreg >> d) & (sreg << d);
      s.vcol[j] = v;
    }
    __syncthreads();

    // -- eroded mask, zeroed final mask, candidates (output columns) ---------
    if (warp < G::NWORD) {
      const int c = tid;  // output column c, stage-0 column c + E
      uint32_t h = s.vcol[c + G::E];
#pragma unroll
      for (int d = 1; d <= G::E; d++)
        h &= s.vcol[c + G::E - d] & s.vcol[c + G::E + d];
      const uint32_t scr1 = h | mreg;
      const int gx = x0 + c;
      const bool inside = gx < width;
      const int widx = (x0 >> 5) + warp;
#pragma unroll
      for (int k = G::E; k < G::E + 8; k++) {
        const int row = newest_v0 - k;
        if (row < y0 || row >= y1)
          continue;
        const bool b = inside && ((scr1 >> k) & 1u);
        const uint32_t word = __ballot_sync(0xffffffffu, b);
        if (lane == 0 && widx < wpr) {
          scr1_bits[(size_t)row * wpr + widx] = word;
          final_bits[(size_t)row * wpr + widx] = 0u;
        }
        if (word == 0u)
          continue;  // warp-uniform
        const uint32_t pk = s.ns[(row - p_first) & (G::RING - 1)][c + G::A];
        const bool cnd = b && !((mreg >> k) & 1u) && (uint64_t)(pk & G::MASK) >= P.p_min;
        const unsigned cm = __ballot_sync(0xffffffffu, cnd);
        if (cm) {
          uint32_t base = 0;
          if (lane == 0)
            base = atomicAdd(&s.ncand, (uint32_t)__popc(cm));
          base = __shfl_sync(0xffffffffu, base, 0);
          if (cnd)
            s.cand[base + __popc(cm & ((1u << lane) - 1u))] =
                (uint32_t)row * (uint32_t)width + (uint32_t)gx;
        }
      }
    }
    __syncthreads();
    if (s.ncand > G::CCAP - G::TW * 8)
      flush_candidates<K>(s, cand, counters, cand_cap);
  }
  __syncthreads();
  flush_candidates<K>(s, cand, counters, cand_cap);
}

// ---------------------------------------------------------------------------
// Segments holding a pixel too large for the packed sums: 32 x 32 tiles of
// the eroded mask with exact 64-bit sums, from the row the streaming block
// stopped at.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(256)
stream_wide(const uint32_t *__restrict__ image, int height, int width,
            const __grid_constant__ LaunchParams P, uint32_t *__restrict__ scr1_bits,
            uint32_t *__restrict__ final_bits, uint32_t *__restrict__ cand,
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
  const int wpr = (width + 31) >> 5;
  for (int i = tid; i <= kMaxN0; i += blockDim.x) {
    rlo[i] = P.root_lo[i];
    rhi[i] = P.root_hi[i];
  }
  const uint32_t nwide = counters[kCtrWide];
  // Work items: (entry, tile column, tile row), tiles of 32 rows from the
  // entry's first row.
  constexpr int TPS = kStreamTW / TS; // tile columns per strip
  constexpr int TPR = (kStreamSH + TS - 1) / TS + 1;
  for (uint32_t item = blockIdx.x; item < nwide * TPS * TPR; item += gridDim.x) {
    const uint4 w = wide_list[item / (TPS * TPR)];
    const int rem = (int)(item % (TPS * TPR));
    const int tcol = rem % TPS, trow = rem / TPS;
    const int tx0 = (int)w.x + tcol * TS;
    const int ty0 = (int)w.y + trow * TS;
    if (ty0 >= (int)w.z || tx0 >= width)
      continue;
    const int ty1 = min((int)w.z, ty0 + TS);
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
    // Eroded mask of the 32 x 32 tile: warp w handles rows w, w + 8, ...
    for (int r = warp; r < TS; r += blockDim.x >> 5) {
      const int gy = ty0 + r;
      const int c = lane;
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
      const bool inside = gy < ty1 && tx0 + c < width;
      const bool b = inside && m;
      const uint32_t word = __ballot_sync(0xffffffffu, b);
      if (lane == 0 && gy < ty1 && (tx0 >> 5) < wpr) {
        scr1_bits[(size_t)gy * wpr + (tx0 >> 5)] = word;
        final_bits[(size_t)gy * wpr + (tx0 >> 5)] = 0u;
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
          cand[g] = (uint32_t)gy * (uint32_t)width + (uint32_t)(tx0 + c);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Stage 2 at the candidates.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(256)
stream_stage2(const uint32_t *__restrict__ image, int height, int width,
              const __grid_constant__ LaunchParams P, const uint32_t *__restrict__ scr1_bits,
              uint32_t *__restrict__ final_bits, const uint32_t *__restrict__ cand,
              uint32_t cand_cap, uint32_t *__restrict__ counters,
              sf_signal_pixel *__restrict__ staging, uint32_t capacity) {
  constexpr int K2 = K + 2;
  const int wpr = (width + 31) >> 5;
  const uint32_t nc = min(counters[kCtrCand], cand_cap);
  const int lane = threadIdx.x & 31;
  for (uint32_t base = blockIdx.x * blockDim.x; base < nc; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    bool sig = false;
    sf_signal_pixel rec;
    uint32_t idx = 0;
    if (i < nc) {
      idx = cand[i];
      const int y = (int)(idx / (uint32_t)width), x = (int)(idx % (uint32_t)width);
      const uint32_t p = __ldg(image + idx);
      uint32_t n = 0;
      unsigned long long S = 0;
      const int ylo = max(0, y - K2), yhi = min(height - 1, y + K2);
      const int xlo = max(0, x - K2), xhi = min(width - 1, x + K2);
      for (int yy = ylo; yy <= yhi; yy++) {
        const uint32_t *row = image + (size_t)yy * width;
        const uint32_t *brow = scr1_bits + (size_t)yy * wpr;
        // The eroded mask over [xlo, xhi] from at most two words.
        const int w0 = xlo >> 5;
        const unsigned long long both =
            (unsigned long long)__ldg(brow + w0) |
            ((w0 + 1 < wpr) ? ((unsigned long long)__ldg(brow + w0 + 1) << 32) : 0ull);
        const unsigned long long bg_bits = ~(both >> (xlo - (w0 << 5)));
        // Row loads issued together, then summed.
        uint32_t v[2 * K2 + 1];
#pragma unroll
        for (int d = 0; d <= 2 * K2; d++)
          v[d] = (xlo + d <= xhi) ? __ldg(row + xlo + d) : 0u;
#pragma unroll
        for (int d = 0; d <= 2 * K2; d++) {
          // Not in the eroded mask (masked pixels are in it), so valid.
          if (xlo + d <= xhi && ((bg_bits >> d) & 1ull)) {
            n++;
            S += v[d];
          }
        }
      }
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
        atomicOr(&final_bits[(size_t)(idx / (uint32_t)width) * wpr + (idx % (uint32_t)width) / 32],
                 1u << ((idx % (uint32_t)width) & 31u));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Ordering: popcounts of the final mask's words, their exclusive scan, then
// each staged record to its ascending position.
// ---------------------------------------------------------------------------
__global__ void order_popc(const uint32_t *__restrict__ bits, const uint32_t *__restrict__ nwords,
                           uint32_t *__restrict__ out) {
  const uint32_t n = *nwords;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = __popc(bits[i]);
}

__global__ void order_scatter(int width, const uint32_t *__restrict__ bits,
                              const uint32_t *__restrict__ prefix,
                              const uint32_t *__restrict__ counters,
                              const sf_signal_pixel *__restrict__ staging, uint32_t capacity,
                              sf_signal_pixel *__restrict__ out) {
  const uint32_t n = min(counters[kCtrTotal], capacity);
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

__global__ void set_word_count(uint32_t *counters, uint32_t nwords) {
  counters[kCtrWords] = nwords;
}

// The caller's count: the signal found, or all ones if the candidate list
// overflowed (the list is then incomplete, as for a count above capacity).
__global__ void finish_count(const uint32_t *counters, uint32_t cand_cap, uint32_t *out) {
  *out = counters[kCtrCand] > cand_cap ? 0xFFFFFFFFu : counters[kCtrTotal];
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

template <int K>
static cudaError_t launch_stream_k(const uint32_t *image, int h, int w, const LaunchParams &P,
                                   const StreamBuffers &b, cudaStream_t stream) {
  using S = StreamSmem<K>;
  static bool configured = false;
  cudaError_t e;
  if (!configured) {
    e = cudaFuncSetAttribute(stream_stage01<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(S));
    if (e != cudaSuccess)
      return e;
    configured = true;
  }
  StreamTables T;
  make_stream_tables(P, &T);
  const int vec = (w % 4 == 0 && reinterpret_cast<uintptr_t>(image) % 16 == 0) ? 1 : 0;
  const dim3 g1((w + kStreamTW - 1) / kStreamTW, (h + kStreamSH - 1) / kStreamSH);
  stream_stage01<K><<<g1, 256, sizeof(S), stream>>>(image, h, w, vec, P, T, b.scr1, b.bits,
                                                     b.cand, b.cand_cap, b.counters, b.wide);
  stream_wide<K><<<2 * 152, 256, 0, stream>>>(image, h, w, P, b.scr1, b.bits, b.cand,
                                               b.cand_cap, b.counters, b.wide);
  stream_stage2<K><<<4 * 152, 256, 0, stream>>>(image, h, w, P, b.scr1, b.bits, b.cand,
                                                 b.cand_cap, b.counters, b.staging,
                                                 b.capacity);
  const uint32_t nwords = (uint32_t)(((size_t)w + 31) / 32 * h);
  order_popc<<<2 * 152, 512, 0, stream>>>(b.bits, b.counters + kCtrWords, b.prefix);
  e = exclusive_scan(b.prefix, b.prefix, b.counters + kCtrWords, nullptr, b.block_sums,
                     nullptr, stream);
  if (e != cudaSuccess)
    return e;
  order_scatter<<<2 * 152, 256, 0, stream>>>(w, b.bits, b.prefix, b.counters, b.staging,
                                             b.capacity, b.out);
  finish_count<<<1, 1, 0, stream>>>(b.counters, b.cand_cap, b.count_out);
  (void)nwords;
  return cudaGetLastError();
}

cudaError_t launch_stream(const uint32_t *image, int h, int w, const LaunchParams &P,
                          const StreamBuffers &b, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(b.counters, 0, kCtrCount * sizeof(uint32_t), stream);
  if (e != cudaSuccess)
    return e;
  const uint32_t nwords = (uint32_t)(((size_t)w + 31) / 32 * h);
  set_word_count<<<1, 1, 0, stream>>>(b.counters, nwords);
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
