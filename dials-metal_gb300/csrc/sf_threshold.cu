// The fused threshold for sm_103a: every stage of src/spots/dext.cc (the
// dispersion test, the erosion, the background-only Poisson test) for one
// output tile per block, from one read of the tile and its halo, with the
// masks kept in shared memory. Then an ordering pass that writes the signal
// list ascending by index, which the reference's device path had to sort on
// the host (src/spots/dext_cuda.cu:855-861).
//
// Per frame, kernel 1 (threshold_tile) writes
//   - the strong-pixel bitmask, one bit per pixel, row-major, ceil(W/32)
//     words per row;
//   - each tile's signal records in tile row-major order into a staging list
//     at a base taken with one atomic per tile;
//   - the tile's base and count, and its count into its tile row's total.
// Kernel 2 (order_signal), one block per tile row, turns the bitmask's
// popcounts into the global row-major position of every record and copies
// the records there; it also leaves the exclusive popcount prefix of every
// bitmask word, so a pixel's position in the list is one lookup and a
// popcount (the labeller's neighbour search).

#include <cuda_runtime.h>
#include <stdint.h>

#include "sf_common.cuh"
#include "sf_threshold.cuh"

namespace sf {

// Tile geometry for a half-width K window and a TW x TH output tile.
template <int K, int TW, int TH> struct Geom {
  static constexpr int E = K - 1;              // erosion radius (dext.cc:117)
  static constexpr int K2 = K + 2;             // stage-2 half-width (dext.cc:165)
  static constexpr int R = K + E + K2;         // total halo, 3K + 1
  static constexpr int IW = TW + 2 * R, IH = TH + 2 * R;  // pixels loaded
  static constexpr int S0W = IW - 2 * K, S0H = IH - 2 * K; // stage-0 results
  static constexpr int S1W = S0W - 2 * E, S1H = S0H - 2 * E; // eroded mask
  static constexpr int O1 = K + E;             // scr1 (0,0) in pixel coords
  static constexpr int NW = TW / 32;           // bitmask words per tile row
  static_assert(TW % 32 == 0, "tile width is whole bitmask words");
  static_assert(S1W == TW + 2 * K2, "erosion region spans the stage-2 window");
};

template <typename T, int K, int TW, int TH> struct Smem {
  using G = Geom<K, TW, TH>;
  using W = typename Traits<T>::W;
  uint32_t pix[G::IH][G::IW];
  W hS[G::IH][G::S0W];          // stage-0 row sums of I; later stage-2 rows
  W hQ[G::IH][G::S0W];          // stage-0 row sums of I^2
  uint8_t hN[G::IH][G::S0W];
  uint8_t scr0[G::S0H][G::S0W];
  uint8_t scr1[G::S1H][G::S1W];
  uint8_t h2N[G::S1H][TW];
  float bg[TH][TW];
  uint16_t pop[TH][TW];
  uint32_t bits[TH][G::NW];
  uint32_t row_prefix[TH * G::NW + 1];
  uint32_t root_lo[kMaxN0 + 1], root_hi[kMaxN0 + 1];
  uint32_t tile_base;
};

template <typename T>
__device__ __forceinline__ bool is_masked(uint32_t v) {
  return v >= Traits<T>::kMasked;
}

template <typename T, int K, int TW, int TH>
__global__ void __launch_bounds__(256)
threshold_tile(const T *__restrict__ image, int height, int width,
               const __grid_constant__ LaunchParams P, uint32_t *__restrict__ bits,
               sf_signal_pixel *__restrict__ staging, uint32_t capacity,
               uint32_t *__restrict__ total, uint32_t *__restrict__ tile_base,
               uint32_t *__restrict__ row_total) {
  using G = Geom<K, TW, TH>;
  using W = typename Traits<T>::W;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem<T, K, TW, TH> &s = *reinterpret_cast<Smem<T, K, TW, TH> *>(smem_raw);

  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  const int tx0 = blockIdx.x * TW, ty0 = blockIdx.y * TH;
  const int x_base = tx0 - G::R, y_base = ty0 - G::R;

  for (int i = tid; i <= kMaxN0; i += nthreads) {
    s.root_lo[i] = P.root_lo[i];
    s.root_hi[i] = P.root_hi[i];
  }

  // Phase 0: the tile and its halo. Pixels off the frame read as masked,
  // which is what the reference's clipped windows and skipped neighbours
  // amount to (dext.cc:71-97, :121-124).
  for (int idx = tid; idx < G::IH * G::IW; idx += nthreads) {
    const int r = idx / G::IW, c = idx - r * G::IW;
    const int gy = y_base + r, gx = x_base + c;
    uint32_t v = Traits<T>::kOutside;
    if (gy >= 0 && gy < height && gx >= 0 && gx < width)
      v = (uint32_t)image[(size_t)gy * width + gx];
    s.pix[r][c] = v;
  }
  __syncthreads();

  // Phase 1: stage-0 row sums of count, I and I^2 over 2K + 1 columns.
  for (int idx = tid; idx < G::IH * G::S0W; idx += nthreads) {
    const int r = idx / G::S0W, c = idx - r * G::S0W;
    uint32_t n = 0;
    W sum = 0, sq = 0;
#pragma unroll
    for (int d = 0; d <= 2 * K; d++) {
      const uint32_t v = s.pix[r][c + d];
      if (!is_masked<T>(v)) {
        n++;
        sum += (W)v;
        sq += (W)v * (W)v;
      }
    }
    s.hN[r][c] = (uint8_t)n;
    s.hS[r][c] = sum;
    s.hQ[r][c] = sq;
  }
  __syncthreads();

  // Phase 2: column sums and the dispersion test; scr0 = signal or masked
  // (dext.cc:111). For the plain dispersion algorithm the full decision is
  // made here at the output pixels.
  for (int idx = tid; idx < G::S0H * G::S0W; idx += nthreads) {
    const int r = idx / G::S0W, c = idx - r * G::S0W;
    uint32_t n = 0;
    W sum = 0, sq = 0;
#pragma unroll
    for (int d = 0; d <= 2 * K; d++) {
      n += s.hN[r + d][c];
      sum += s.hS[r + d][c];
      sq += s.hQ[r + d][c];
    }
    bool sig;
    if constexpr (sizeof(T) == 4)
      sig = stage0_u32(n, sum, sq, P, s.root_lo, s.root_hi);
    else
      sig = stage0_u16(n, (uint32_t)sum, (uint32_t)sq, P);
    const uint32_t v = s.pix[r + K][c + K];
    s.scr0[r][c] = (sig || is_masked<T>(v)) ? 1 : 0;

    if (P.algorithm == SF_DISPERSION) {
      const int orow = r + K - G::R, ocol = c + K - G::R;
      if (orow >= 0 && orow < TH && ocol >= 0 && ocol < TW) {
        bool strong = false;
        float bg = 0.0f;
        if (sig && !is_masked<T>(v) && v >= P.p_min) {
          // (m p - s) > sigma_s sqrt(g s m), in the pixel type's real type.
          if constexpr (sizeof(T) == 4) {
            const double m = (double)n, sd = __ull2double_rn(sum), pv = (double)v;
            strong = __dsub_rn(__dmul_rn(m, pv), sd) >
                     __dmul_rn(P.sigma_s, __dsqrt_rn(__dmul_rn(__dmul_rn(P.gain, sd), m)));
            bg = __double2float_rn(__ddiv_rn(sd, m));
          } else {
            const float m = __uint2float_rn(n), sd = __uint2float_rn((uint32_t)sum),
                        pv = __uint2float_rn(v);
            strong = __fsub_rn(__fmul_rn(m, pv), sd) >
                     __fmul_rn((float)P.sigma_s,
                               __fsqrt_rn(__fmul_rn(__fmul_rn((float)P.gain, sd), m)));
            bg = __fdiv_rn(sd, m);
          }
        }
        s.bg[orow][ocol] = strong ? bg : -1.0f;
        s.pop[orow][ocol] = (uint16_t)n;
      }
    }
  }
  __syncthreads();

  if (P.algorithm == SF_DISPERSION_EXTENDED) {
    // Phase 3: erode by K - 1; masked pixels are set (dext.cc:117-142).
    for (int idx = tid; idx < G::S1H * G::S1W; idx += nthreads) {
      const int r = idx / G::S1W, c = idx - r * G::S1W;
      const uint32_t v = s.pix[r + G::O1][c + G::O1];
      uint8_t m = 1;
      if (!is_masked<T>(v)) {
        m = s.scr0[r + G::E][c + G::E];
        for (int dr = 0; dr <= 2 * G::E && m; dr++)
          for (int dc = 0; dc <= 2 * G::E; dc++)
            if (!s.scr0[r + dr][c + dc]) {
              m = 0;
              break;
            }
      }
      s.scr1[r][c] = m;
    }
    __syncthreads();

    // Phase 4: stage-2 row sums over the background (valid and not eroded;
    // masked pixels are in scr1, dext.cc:151-161). Reuses hS.
    W(*h2S)[G::S0W] = s.hS;
    for (int idx = tid; idx < G::S1H * TW; idx += nthreads) {
      const int r = idx / TW, c = idx - r * TW;
      uint32_t n = 0;
      W sum = 0;
#pragma unroll
      for (int d = 0; d <= 2 * G::K2; d++) {
        if (!s.scr1[r][c + d]) {
          n++;
          sum += (W)s.pix[r + G::O1][c + G::O1 + d];
        }
      }
      s.h2N[r][c] = (uint8_t)n;
      h2S[r][c] = sum;
    }
    __syncthreads();

    // Phase 5: column sums and the Poisson test at candidates (dext.cc:165-222).
    for (int idx = tid; idx < TH * TW; idx += nthreads) {
      const int r = idx / TW, c = idx - r * TW;
      const uint32_t v = s.pix[r + G::R][c + G::R];
      const bool cand = !is_masked<T>(v) && v >= P.p_min && s.scr1[r + G::K2][c + G::K2];
      float bg = -1.0f;
      uint32_t n = 0;
      if (cand) {
        W sum = 0;
        for (int d = 0; d <= 2 * G::K2; d++) {
          n += s.h2N[r + d][c];
          sum += h2S[r + d][c];
        }
        float b;
        bool sig;
        if constexpr (sizeof(T) == 4)
          sig = stage2_u32(v, n, sum, P, &b);
        else
          sig = stage2_u16(v, n, (uint32_t)sum, P, &b);
        if (sig)
          bg = b;
      }
      s.bg[r][c] = bg;
      s.pop[r][c] = (uint16_t)n;
    }
    __syncthreads();
  }

  // Phase 6: bitmask words by warp ballot (a warp per 32-column word).
  const int lane = tid & 31, warp = tid >> 5, nwarps = nthreads >> 5;
  for (int w = warp; w < TH * G::NW; w += nwarps) {
    const int r = w / G::NW, word = w - r * G::NW;
    const int c = word * 32 + lane;
    const int gy = ty0 + r, gx = tx0 + c;
    const bool inside = gy < height && gx < width;
    const bool sig = inside && s.bg[r][c] >= 0.0f;
    const uint32_t b = __ballot_sync(0xffffffffu, sig);
    if (lane == 0)
      s.bits[r][word] = b;
  }
  __syncthreads();

  // Phase 7: tile-local prefix over the words in row-major order, one atomic
  // for the tile's place in the staging list.
  if (warp == 0) {
    constexpr int NWORDS = TH * G::NW;
    uint32_t carry = 0;
    for (int base = 0; base < NWORDS; base += 32) {
      const int i = base + lane;
      const uint32_t cnt = i < NWORDS ? __popc((&s.bits[0][0])[i]) : 0;
      uint32_t incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
          incl += t;
      }
      if (i < NWORDS)
        s.row_prefix[i] = carry + incl - cnt;
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) {
      s.row_prefix[NWORDS] = carry;
      const uint32_t base = carry ? atomicAdd(total, carry) : 0u;
      s.tile_base = base;
      const uint32_t tile = blockIdx.y * gridDim.x + blockIdx.x;
      tile_base[tile] = base;
      if (carry)
        atomicAdd(&row_total[blockIdx.y], carry);
    }
  }
  __syncthreads();

  // Phase 8: the records, and the bitmask words.
  const int words_per_row = (width + 31) >> 5;
  const uint32_t tbase = s.tile_base;
  for (int w = warp; w < TH * G::NW; w += nwarps) {
    const int r = w / G::NW, word = w - r * G::NW;
    const int gy = ty0 + r;
    if (gy >= height)
      continue;
    const uint32_t b = s.bits[r][word];
    const int gword = (tx0 >> 5) + word;
    if (lane == 0 && gword < words_per_row)
      bits[(size_t)gy * words_per_row + gword] = b;
    if ((b >> lane) & 1u) {
      const int c = word * 32 + lane;
      const uint32_t slot = tbase + s.row_prefix[w] + __popc(b & ((1u << lane) - 1u));
      if (slot < capacity) {
        sf_signal_pixel px;
        px.index = (uint32_t)gy * (uint32_t)width + (uint32_t)(tx0 + c);
        px.value = s.pix[r + G::R][c + G::R];
        px.background = s.bg[r][c];
        px.population = s.pop[r][c];
        px.reserved = 0;
        staging[slot] = px;
      }
    }
  }
}

// Kernel 2: one block per tile row. Global position of each bitmask word's
// records = (signal in earlier tile rows) + (row-major prefix inside this
// tile row); staging position = the tile's base + its tile-local prefix.
template <int TW, int TH>
__global__ void __launch_bounds__(512)
order_signal(int height, int width, const uint32_t *__restrict__ bits,
             const sf_signal_pixel *__restrict__ staging, uint32_t capacity,
             const uint32_t *__restrict__ tile_base,
             const uint32_t *__restrict__ row_total, sf_signal_pixel *__restrict__ out,
             uint32_t *__restrict__ word_prefix) {
  constexpr int NW = TW / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int words_per_row = (width + 31) >> 5;
  const int tiles_x = (width + TW - 1) / TW;
  const int R = blockIdx.x;
  const int y0 = R * TH;
  const int rows = min(TH, height - y0);
  const int nwords = rows * words_per_row;
  uint32_t *cnt = reinterpret_cast<uint32_t *>(smem_raw);       // nwords
  uint32_t *tile_pre = cnt + TH * words_per_row;                  // nwords
  __shared__ uint32_t s_warp[32], s_warp_excl[32];
  __shared__ uint32_t s_base, s_chunk;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;

  // Signal in earlier tile rows.
  uint32_t acc = 0;
  for (int i = tid; i < R; i += blockDim.x)
    acc += row_total[i];
  for (int o = 16; o; o >>= 1)
    acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0)
    s_warp[warp] = acc;
  for (int i = tid; i < nwords; i += blockDim.x)
    cnt[i] = __popc(bits[(size_t)y0 * words_per_row + i]);
  __syncthreads();
  if (tid == 0) {
    uint32_t t = 0;
    for (int i = 0; i < nwarps; i++)
      t += s_warp[i];
    s_base = t;
  }
  __syncthreads();

  // Tile-local prefix: per tile column, row-major over its NW-word rows.
  for (int tc = tid; tc < tiles_x; tc += blockDim.x) {
    uint32_t run = 0;
    for (int r = 0; r < rows; r++)
      for (int k = 0; k < NW; k++) {
        const int wc = tc * NW + k;
        if (wc < words_per_row) {
          tile_pre[r * words_per_row + wc] = run;
          run += cnt[r * words_per_row + wc];
        }
      }
  }
  __syncthreads();

  // Row-major exclusive scan of cnt, in place, one block-wide chunk at a time.
  uint32_t carry = 0;
  for (int base = 0; base < nwords; base += blockDim.x) {
    const int i = base + tid;
    const uint32_t v = i < nwords ? cnt[i] : 0u;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o)
        incl += t;
    }
    if (lane == 31)
      s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const uint32_t wv = lane < nwarps ? s_warp[lane] : 0u;
      uint32_t wi = wv;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o)
          wi += t;
      }
      if (lane < nwarps)
        s_warp_excl[lane] = wi - wv;
      if (lane == 31)
        s_chunk = wi;
    }
    __syncthreads();
    if (i < nwords)
      cnt[i] = carry + s_warp_excl[warp] + incl - v;
    carry += s_chunk;
    __syncthreads();
  }

  // Copy records into place.
  const uint32_t gbase = s_base;
  for (int i = tid; i < nwords; i += blockDim.x) {
    const int r = i / words_per_row, wc = i - r * words_per_row;
    const uint32_t b = bits[(size_t)y0 * words_per_row + i];
    const uint32_t dst = gbase + cnt[i];
    if (word_prefix)
      word_prefix[(size_t)y0 * words_per_row + i] = dst;
    if (!b)
      continue;
    const int tc = wc / NW;
    const uint32_t src = tile_base[R * tiles_x + tc] + tile_pre[i];
    const int n = __popc(b);
    for (int j = 0; j < n; j++) {
      if (src + j < capacity && dst + j < capacity)
        out[dst + j] = staging[src + j];
    }
  }
  (void)height;
}

// ---------------------------------------------------------------------------
// Host-side launch.
// ---------------------------------------------------------------------------

template <typename T, int K>
static cudaError_t launch_k(const T *image, int h, int w, const LaunchParams &P,
                            const FrameBuffers &fb, cudaStream_t stream) {
  constexpr int TW = kTileW, TH = kTileH;
  using S = Smem<T, K, TW, TH>;
  const size_t smem = sizeof(S);
  static bool configured = false; // per instantiation; attribute is per device
  cudaError_t e = cudaSuccess;
  if (!configured) {
    e = cudaFuncSetAttribute(threshold_tile<T, K, TW, TH>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
      return e;
    configured = true;
  }
  const dim3 grid((w + TW - 1) / TW, (h + TH - 1) / TH);
  threshold_tile<T, K, TW, TH><<<grid, 256, smem, stream>>>(
      image, h, w, P, fb.bits, fb.staging, fb.capacity, fb.total, fb.tile_base,
      fb.row_total);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return e;
  const size_t smem2 = order_smem_bytes(w);
  if (smem2 > 48 * 1024) {
    e = cudaFuncSetAttribute(order_signal<TW, TH>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
    if (e != cudaSuccess)
      return e;
  }
  order_signal<TW, TH><<<grid.y, 512, smem2, stream>>>(
      h, w, fb.bits, fb.staging, fb.capacity, fb.tile_base, fb.row_total, fb.out,
      fb.word_prefix);
  return cudaGetLastError();
}

size_t order_smem_bytes(int width) {
  return 2 * sizeof(uint32_t) * (size_t)kTileH * ((width + 31) / 32);
}

template <typename T>
cudaError_t launch_threshold(const T *image, int h, int w, const LaunchParams &P,
                             const FrameBuffers &fb, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(fb.total, 0, sizeof(uint32_t), stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(fb.row_total, 0, sizeof(uint32_t) * tiles_y(h), stream);
  if (e != cudaSuccess)
    return e;
  switch (P.half) {
  case 2:
    return launch_k<T, 2>(image, h, w, P, fb, stream);
  case 3:
    return launch_k<T, 3>(image, h, w, P, fb, stream);
  case 4:
    return launch_k<T, 4>(image, h, w, P, fb, stream);
  default:
    return cudaErrorInvalidValue;
  }
}

template cudaError_t launch_threshold<uint32_t>(const uint32_t *, int, int,
                                                const LaunchParams &,
                                                const FrameBuffers &, cudaStream_t);
template cudaError_t launch_threshold<uint16_t>(const uint16_t *, int, int,
                                                const LaunchParams &,
                                                const FrameBuffers &, cudaStream_t);

} // namespace sf
