// Frame decompression on the device (sf_decompress.cuh).
//
// k_decode gives each block of a chunk to one warp:
//
//   LZ4     every lane follows the same parse of the block, a 32-byte
//           window of input (a byte a lane) at a time: each lane reads the
//           sequence that would start at its byte, and the short sequences
//           chained from the window's start are taken together, their
//           literals written at once by the lanes that hold them. Matches are
//           copied by the lanes together, a byte or (long ones, 32-bit
//           pixels) a word a lane. A match whose offset is shorter than its
//           length repeats a pattern of `offset` bytes: a one-byte run is
//           filled with 16-byte stores, other patterns are copied in passes
//           of D bytes from D back, D doubling from the offset, so that no
//           pass reads what it writes.
//   planes  a bitshuffle block decodes into the warp's 8 KB of shared memory
//           (bitshuffle's default block is 8192 bytes); for each group of 8
//           elements and each byte j of an element, the group's byte of each
//           of the 8 planes 8j .. 8j + 7 forms an 8 x 8 bit matrix whose
//           transpose holds byte j of the 8 elements. A lane takes 4 groups
//           at a time, reading each plane's 4 bytes as one word. Larger
//           blocks decode into a frame-sized scratch buffer instead.
//
// The host has already checked the framing (every block lies inside the
// chunk); the device checks each LZ4 stream as LZ4_decompress_safe does and
// records the first block that fails.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdio>
#include <cstring>

#include "sf_api.h"
#include "sf_decompress.cuh"
#include "sf_stream.cuh"

namespace sf {
namespace {

constexpr int kDecWarps = 4;
constexpr uint32_t kDecBuf = 8192;  // bytes of a warp's decoded block
constexpr size_t kDecMaxIn = size_t(1) << 31;  // a block's compressed bytes, below

__device__ __forceinline__ void prefetch_l1(const void *p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// dst[0, n) = v by the warp: bytes up to a 16-byte boundary, 16-byte
// stores, the bytes after the last whole 16.
template <typename Out>
__device__ __forceinline__ void fill_warp(Out *dst, uint8_t v, uint32_t n, int lane) {
  const uint32_t head = min(n, (uint32_t)(-(uintptr_t)dst & 15u));
  const uint32_t body = (n - head) & ~15u;
  if ((uint32_t)lane < head)
    dst[lane] = v;
  const uint32_t word = v * 0x01010101u;
  const uint4 w4 = make_uint4(word, word, word, word);
  uint4 *body4 = reinterpret_cast<uint4 *>(dst + head);
  for (uint32_t i = lane; i < body / 16; i += 32)
    body4[i] = w4;
  const uint32_t tail = n - head - body;
  if ((uint32_t)lane < tail)
    dst[head + body + lane] = v;
  __syncwarp();
}

// dst[op, op + m) = dst[op - D, op - D + m) for m <= D (so that no byte it
// reads is one it writes), by the warp, a byte a lane. With kWords, past 32
// bytes a lane writes a 32-bit word at a time: the bytes up to a 4-byte
// boundary, the words (each from the two source words it straddles, by a
// funnel shift), the bytes after the last whole word. The word reads may
// take up to 2 bytes past the source, which the shift drops.
template <bool kWords, typename Out>
__device__ __forceinline__ void copy_pass(Out *dst, uint32_t op, uint32_t D, uint32_t m,
                                          int lane) {
  Out *d = dst + op;
  if (!kWords) {
    for (uint32_t i = lane; i < m; i += 32)
      d[i] = d[(int)i - (int)D];
    return;
  }
  if (m <= 32) {
    if ((uint32_t)lane < m)
      d[lane] = d[(int)lane - (int)D];
    return;
  }
  const uint32_t head = (uint32_t)(-(uintptr_t)d) & 3u;
  if ((uint32_t)lane < head)
    d[lane] = d[(int)lane - (int)D];
  const uint32_t nw = (m - head) >> 2;
  uint32_t *dw = reinterpret_cast<uint32_t *>(d + head);
  const Out *s = d + head - D;
  const uint32_t sh = (uint32_t)(uintptr_t)s & 3u;
  const uint32_t *sw = reinterpret_cast<const uint32_t *>(s - sh);
  if (sh == 0) {
    for (uint32_t i = lane; i < nw; i += 32)
      dw[i] = sw[i];
  } else {
    for (uint32_t i = lane; i < nw; i += 32)
      dw[i] = __funnelshift_r(sw[i], sw[i + 1], 8u * sh);
  }
  const uint32_t t0 = head + 4u * nw;
  if ((uint32_t)lane < m - t0)
    d[t0 + lane] = d[(int)(t0 + lane) - (int)D];
}

// dst[op, op + ml) = the match at `off` back, by the warp. A match that
// overlaps what it writes (off < ml) repeats a pattern of `off` bytes: runs
// of one byte are filled; otherwise it goes in passes of D bytes from D back,
// D doubling from off up to kPass, so that no pass reads what it writes.
template <bool kWords, typename Out>
__device__ __forceinline__ void copy_match(Out *dst, uint32_t op, uint32_t off, uint32_t ml,
                                           int lane) {
  constexpr uint32_t kPass = kWords ? 512u : 128u;
  if (off >= ml) {
    copy_pass<kWords>(dst, op, off, ml, lane);
    __syncwarp();
    return;
  }
  if (off == 1) {
    fill_warp(dst + op, dst[op - 1], ml, lane);
    return;
  }
  uint32_t D = off, done = 0;
  while (done < ml) {
    const uint32_t m = min(ml - done, min(D, kPass));
    copy_pass<kWords>(dst, op + done, D, m, lane);
    __syncwarp();
    done += m;
    if (m == D && D < kPass)
      D *= 2;
  }
}

// One LZ4 block in[0, n) into dst[0, cap) by the whole warp. Returns the
// bytes produced, or minus (the input position where the stream was found
// bad) minus 1. The checks are LZ4_decompress_safe's: a literal run that
// reaches the last 12 bytes of output or the last 8 of input must end the
// block at the input's end; a match must start inside the output and end
// before its last 5 bytes.
//
// The parse goes a window at a time: one load of the next 32 input bytes, a
// byte a lane. Every lane reads the sequence that would start at its byte
// (token, offset, length); the sequences that chain from the window's first
// byte and lie inside it, with a literal run under 15 bytes and a match
// length of at most one extra byte (most of them), are taken together: their
// output positions as the chain is walked, the checks by each sequence's
// lane, all their literals written at once from the lanes that hold them,
// then their matches in order. A window whose first sequence is not of that
// kind, or would fail a check, takes the byte-by-byte parse for that
// sequence, which reports the error.
template <bool kWords, typename Out>
__device__ __forceinline__ long long lz4_warp(const uint8_t *__restrict__ in, uint32_t n,
                                              Out *dst, uint32_t cap, int lane) {
  uint32_t ip = 0, op = 0;
  for (;;) {
    if (ip >= n)
      return -(long long)ip - 1;
    // (n < 2^31, so that ip + lane cannot wrap: the host refuses larger blocks.)
    const uint32_t w = ip + lane < n ? (uint32_t)__ldg(in + ip + lane) : 0u;
    {
      // The sequence a token at this lane's byte would start.
      const uint32_t l0 = w >> 4, nib = w & 15u;
      const uint32_t off = __shfl_sync(~0u, w, lane + l0 + 1) |
                           __shfl_sync(~0u, w, lane + l0 + 2) << 8;
      const uint32_t e = __shfl_sync(~0u, w, lane + l0 + 3);
      const uint32_t ext = nib == 15u ? 1u : 0u;
      const uint32_t len = l0 + 3u + ext;  // its bytes
      const uint32_t ml = nib + 4u + (ext ? e : 0u);
      const bool fits = l0 < 15u && (uint32_t)lane + len <= 32u && !(ext && e == 255u);
      // The chain of such sequences from the window's first byte, and the
      // output before each (its lane keeps it).
      const uint32_t step = fits ? len | (l0 + ml) << 8 : 0u;
      uint32_t toks = 0, acc = 0, before = 0;
      for (uint32_t p = 0; p < 32u;) {  // warp-uniform
        const uint32_t s = __shfl_sync(~0u, step, p);
        if (s == 0)
          break;
        toks |= 1u << p;
        if ((uint32_t)lane == p)
          before = acc;
        acc += s >> 8;
        p += s & 0xFFu;
      }
      const bool tok = (toks >> lane) & 1u;
      const unsigned long long at = (unsigned long long)op + before;
      // Not the last sequence (its literals end 12 bytes before the output's
      // end and 8 before the input's), the offset inside the output, the
      // match ending 5 bytes before the output's end.
      const bool ok = !tok || (at + l0 + 12 <= cap &&
                               (unsigned long long)ip + lane + l0 + 9 <= n && off != 0 &&
                               off <= at + l0 && at + l0 + ml + 5 <= cap);
      const uint32_t bad = __ballot_sync(~0u, !ok);
      const uint32_t keep = toks & ((bad & (0u - bad)) - 1u);  // those before the first bad
      if (keep) {
        // Each lane's byte against the last kept token at or below it.
        const uint32_t below = keep & ((2u << lane) - 1u);
        const int t = 31 - __clz(below);
        const uint32_t tl = __shfl_sync(~0u, l0, t & 31);
        const uint32_t to = __shfl_sync(~0u, (uint32_t)at, t & 31);
        const uint32_t r = (uint32_t)(lane - t - 1);
        if (below && r < tl)
          dst[to + r] = (Out)w;
        __syncwarp();
        const uint32_t mo = (uint32_t)at + l0, mp = off | ml << 16;
        for (uint32_t m = keep; m; m &= m - 1u) {  // warp-uniform
          const int k = __ffs(m) - 1;
          const uint32_t o = __shfl_sync(~0u, mo, k), q = __shfl_sync(~0u, mp, k);
          copy_match<kWords>(dst, o, q & 0xFFFFu, q >> 16, lane);
        }
        const int last = 31 - __clz(keep);
        ip += (uint32_t)last + __shfl_sync(~0u, len, last);
        op = __shfl_sync(~0u, mo + ml, last);
        continue;
      }
    }
    const uint32_t token = __shfl_sync(~0u, w, 0);
    ip++;
    uint32_t lit = token >> 4;
    if (lit == 15) {
      uint32_t s;
      do {
        if (ip >= n)
          return -(long long)ip - 1;
        s = __ldg(in + ip++);
        lit += s;
      } while (s == 255);
    }
    const bool last = (unsigned long long)op + lit + 12 > cap ||
                      (unsigned long long)ip + lit + 8 > n;
    if (last && ((unsigned long long)ip + lit != n || (unsigned long long)op + lit > cap))
      return -(long long)ip - 1;
    for (uint32_t i = lane; i < lit; i += 32)
      dst[op + i] = __ldg(in + ip + i);
    ip += lit;
    op += lit;
    __syncwarp();
    if (last)
      return op;
    const uint32_t off = __ldg(in + ip) | (uint32_t)__ldg(in + ip + 1) << 8;
    ip += 2;
    if (off == 0 || off > op)
      return -(long long)ip - 1;
    uint32_t ml = token & 15u;
    if (ml == 15) {
      uint32_t s;
      do {
        if (ip >= n)
          return -(long long)ip - 1;
        s = __ldg(in + ip++);
        if (ip + 5 > n)
          return -(long long)ip - 1;
        ml += s;
      } while (s == 255);
    }
    ml += 4;
    if ((unsigned long long)op + ml + 5 > cap)
      return -(long long)ip - 1;
    copy_match<kWords>(dst, op, off, ml, lane);
    op += ml;
  }
}

// x holds an 8 x 8 bit matrix, row r in byte r (bit c = column c); returns
// its transpose, by three exchanges of off-diagonal blocks (1 x 1 within
// 2 x 2, 2 x 2 within 4 x 4, 4 x 4 within 8 x 8).
__device__ __forceinline__ unsigned long long transpose8(unsigned long long x) {
  unsigned long long t;
  t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull;
  x ^= t ^ (t << 7);
  t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull;
  x ^= t ^ (t << 14);
  t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull;
  x ^= t ^ (t << 28);
  return x;
}

// The n elements (a multiple of 8) of E bytes of one bitshuffle block from
// its planes (plane r at planes + r * n / 8) to dst, 16-byte aligned.
template <int E, typename In>
__device__ __forceinline__ void unshuffle(const In *planes, uint32_t n, uint8_t *dst, int lane) {
  const uint32_t row = n >> 3;
  for (uint32_t g = lane; g < row; g += 32) {
    uint32_t e[8];
#pragma unroll
    for (int t = 0; t < 8; t++)
      e[t] = 0;
#pragma unroll
    for (int j = 0; j < E; j++) {
      unsigned long long x = 0;
#pragma unroll
      for (int k = 0; k < 8; k++)
        x |= (unsigned long long)(uint8_t)planes[(8 * j + k) * row + g] << (8 * k);
      x = transpose8(x);
#pragma unroll
      for (int t = 0; t < 8; t++)
        e[t] |= (uint32_t)((x >> (8 * t)) & 0xFFu) << (8 * j);
    }
    if (E == 4) {
      uint4 *o = reinterpret_cast<uint4 *>(dst + 32 * (size_t)g);
      o[0] = make_uint4(e[0], e[1], e[2], e[3]);
      o[1] = make_uint4(e[4], e[5], e[6], e[7]);
    } else {
      *reinterpret_cast<uint4 *>(dst + 16 * (size_t)g) =
          make_uint4(e[0] | e[1] << 16, e[2] | e[3] << 16, e[4] | e[5] << 16, e[6] | e[7] << 16);
    }
  }
}

// 4 x 4 byte transpose: byte t of out[i] = byte i of in[t].
__device__ __forceinline__ void bytes4x4(uint32_t a, uint32_t b, uint32_t c, uint32_t d,
                                         uint32_t out[4]) {
  const uint32_t ab0 = __byte_perm(a, b, 0x5140), ab1 = __byte_perm(a, b, 0x7362);
  const uint32_t cd0 = __byte_perm(c, d, 0x5140), cd1 = __byte_perm(c, d, 0x7362);
  out[0] = __byte_perm(ab0, cd0, 0x5410);
  out[1] = __byte_perm(ab0, cd0, 0x7632);
  out[2] = __byte_perm(ab1, cd1, 0x5410);
  out[3] = __byte_perm(ab1, cd1, 0x7632);
}

// The 8 x 8 bit transpose of transpose8 on the two halves of x (lo: rows
// 0-3, hi: rows 4-7): the first two exchanges stay within a half.
__device__ __forceinline__ void transpose8_halves(uint32_t &lo, uint32_t &hi) {
  uint32_t t;
  t = (lo ^ (lo >> 7)) & 0x00AA00AAu;
  lo ^= t ^ (t << 7);
  t = (hi ^ (hi >> 7)) & 0x00AA00AAu;
  hi ^= t ^ (t << 7);
  t = (lo ^ (lo >> 14)) & 0x0000CCCCu;
  lo ^= t ^ (t << 14);
  t = (hi ^ (hi >> 14)) & 0x0000CCCCu;
  hi ^= t ^ (t << 14);
  t = (lo ^ (hi << 4)) & 0xF0F0F0F0u;
  lo ^= t;
  hi ^= t >> 4;
}

// unshuffle for planes in shared memory whose rows are whole 32-bit words
// (n a multiple of 32): a lane takes 4 groups (32 elements) at a time, the
// 8 planes of each element byte read as one word each.
template <int E>
__device__ __forceinline__ void unshuffle_words(const uint8_t *planes, uint32_t n, uint8_t *dst,
                                                int lane) {
  const uint32_t row = n >> 3;
  for (uint32_t q = lane; q < row / 4; q += 32) {
    uint32_t lo[E][4], hi[E][4];
#pragma unroll
    for (int j = 0; j < E; j++) {
      uint32_t w[8];
#pragma unroll
      for (int k = 0; k < 8; k++)
        w[k] = *reinterpret_cast<const uint32_t *>(planes + (8 * j + k) * row + 4 * q);
      bytes4x4(w[0], w[1], w[2], w[3], lo[j]);
      bytes4x4(w[4], w[5], w[6], w[7], hi[j]);
#pragma unroll
      for (int t = 0; t < 4; t++)
        transpose8_halves(lo[j][t], hi[j][t]);
    }
    // Group 4q + t: byte t' of lo[j][t] (hi for t' >= 4) is byte j of its
    // element t'.
#pragma unroll
    for (int t = 0; t < 4; t++) {
      if (E == 4) {
        uint32_t a[4], b[4];
        bytes4x4(lo[0][t], lo[1 % E][t], lo[2 % E][t], lo[3 % E][t], a);
        bytes4x4(hi[0][t], hi[1 % E][t], hi[2 % E][t], hi[3 % E][t], b);
        uint4 *o = reinterpret_cast<uint4 *>(dst + 32 * (size_t)(4 * q + t));
        o[0] = make_uint4(a[0], a[1], a[2], a[3]);
        o[1] = make_uint4(b[0], b[1], b[2], b[3]);
      } else {
        *reinterpret_cast<uint4 *>(dst + 16 * (size_t)(4 * q + t)) =
            make_uint4(__byte_perm(lo[0][t], lo[1 % E][t], 0x5140),
                       __byte_perm(lo[0][t], lo[1 % E][t], 0x7362),
                       __byte_perm(hi[0][t], hi[1 % E][t], 0x5140),
                       __byte_perm(hi[0][t], hi[1 % E][t], 0x7362));
      }
    }
  }
}

__device__ __forceinline__ void report(uint32_t *status, uint32_t kind, uint32_t block,
                                       long long code, int lane) {
  if (lane == 0 && atomicCAS(status, 0u, kind) == 0u) {
    status[1] = block;
    status[2] = (uint32_t)(int32_t)code;
  }
}

template <int E>
__global__ void __launch_bounds__(kDecWarps * 32)
k_decode(const uint8_t *__restrict__ in, const DecodeBlock *__restrict__ blocks,
         uint32_t nblocks, uint8_t *__restrict__ out, uint8_t *__restrict__ scratch,
         uint32_t *__restrict__ status, uint32_t *__restrict__ next) {
  __shared__ __align__(16) uint8_t buf[kDecWarps][kDecBuf];
  // Word copies pay on the planes of 32-bit pixels (long repeats between
  // planes); on those of 16-bit pixels byte copies measured faster.
  constexpr bool kWords = E == 4;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // Blocks are taken in turn from one counter: a warp that finishes early
  // takes the next, so that blocks of uneven cost even out.
  auto take = [&]() {
    uint32_t b = 0;
    if (lane == 0)
      b = atomicAdd(next, 1u);
    return __shfl_sync(0xffffffffu, b, 0);
  };
  for (uint32_t b = take(); b < nblocks; b = take()) {
    const DecodeBlock d = blocks[b];
    const uint8_t *src = in + d.in_off;
    uint8_t *dst = out + d.out_off;
    if (d.mode == kDecRaw) {
      for (uint32_t i = lane; i < d.in_bytes; i += 32)
        dst[i] = src[i];
      continue;
    }
    // The parse reads the block's bytes one dependent load at a time: have
    // its lines in L1 first.
    for (uint32_t i = (uint32_t)lane * 128u; i < d.in_bytes; i += 32u * 128u)
      prefetch_l1(src + i);
    if (d.mode == kDecLz4) {
      const long long r = lz4_warp<true>(src, d.in_bytes, dst, d.out_bytes, lane);
      if (r < 0)
        report(status, kDecBad, b, r, lane);
      else if (r != (long long)d.out_bytes)
        report(status, kDecShort, b, r, lane);
      continue;
    }
    long long r;
    if (d.out_bytes <= kDecBuf) {
      r = lz4_warp<kWords>(src, d.in_bytes, buf[warp], d.out_bytes, lane);
      if (r == (long long)d.out_bytes) {
        if (d.elems % 32 == 0)
          unshuffle_words<E>(buf[warp], d.elems, dst, lane);
        else
          unshuffle<E>(buf[warp], d.elems, dst, lane);
      }
    } else {
      uint8_t *tmp = scratch + d.out_off;
      r = lz4_warp<kWords>(src, d.in_bytes, tmp, d.out_bytes, lane);
      if (r == (long long)d.out_bytes)
        unshuffle<E>(tmp, d.elems, dst, lane);
    }
    if (r != (long long)d.out_bytes)
      report(status, kDecBad, b, -91, lane);  // bitshuffle's code for a bad block
    __syncwarp();  // the buffer is free for the warp's next block
  }
}

uint32_t be32(const uint8_t *p) {
  return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3];
}

int bad_data(const std::string &text) {
  t_last_error = text;
  return SF_EDATA;
}

}  // namespace

int plan_chunk(const uint8_t *data, size_t nbytes, const char *algorithm, unsigned bit_depth,
               size_t height, size_t width, size_t out_bytes, ChunkPlan *plan) {
  plan->blocks.clear();
  plan->scratch = false;
  // decompress.cc:80-84
  const size_t expected = height * width * bit_depth / 8;
  const size_t element = bit_depth / 8;
  if (element == 0 || out_bytes < expected)
    return bad_data("output buffer too small for the frame");
  plan->frame_bytes = expected;
  plan->element = (unsigned)element;
  char text[256];
  if (!algorithm || !algorithm[0]) {  // decompress.cc:86-94
    plan->algorithm = kChunkNone;
    plan->payload = nbytes;
    if (nbytes != expected) {
      std::snprintf(text, sizeof text, "uncompressed frame is %zu bytes, expected %zu", nbytes,
                    expected);
      return bad_data(text);
    }
    return SF_OK;
  }
  // decompress.cc:96-109: the 12-byte filter header.
  if (!data || nbytes < 12)
    return bad_data("too short for a filter header");
  unsigned long long usize = 0;
  for (int i = 0; i < 8; i++)
    usize = usize << 8 | data[i];
  const uint32_t block = be32(data + 8);
  if (usize != expected) {
    std::snprintf(text, sizeof text, "filter header says %llu bytes uncompressed, expected %zu",
                  usize, expected);
    return bad_data(text);
  }
  const uint8_t *p = data + 12;
  const size_t n = nbytes - 12;
  plan->payload = n;
  if (!std::strcmp(algorithm, "bslz4")) {
    // bshuf_decompress_lz4(payload, out, expected / element, element,
    // block / element) (decompress.cc:113-121), its blocks walked here.
    plan->algorithm = kChunkBitshuffle;
    if (element != 2 && element != 4) {
      std::snprintf(text, sizeof text,
                    "bitshuffle frames of %u-bit pixels are not decoded on the device",
                    bit_depth);
      t_last_error = text;
      return SF_EUNSUPPORTED;
    }
    size_t bs = block / element;
    if (bs == 0)
      bs = std::max<size_t>(8192 / element / 8 * 8, 128);  // bitshuffle's default
    if (bs % 8)
      return bad_data("bitshuffle decompression failed with code -81");
    const size_t size = expected / element;
    const size_t nfull = size / bs;
    size_t last = size % bs;
    last -= last % 8;
    size_t ip = 0, op = 0;
    plan->blocks.reserve(nfull + 2);
    for (size_t b = 0; b < nfull + (last ? 1 : 0); b++) {
      const size_t elems = b < nfull ? bs : last;
      if (n - ip < 4)
        return bad_data("bitshuffle decompression failed with code -1");
      const size_t c = be32(p + ip);
      ip += 4;
      if (c > n - ip)
        return bad_data("bitshuffle decompression failed with code -1");
      if (elems * element > 0xFFFFFFFFull || c >= kDecMaxIn) {
        t_last_error = "bitshuffle blocks of 4 GB or more (2 GB compressed) are not decoded "
                       "on the device";
        return SF_EUNSUPPORTED;
      }
      plan->blocks.push_back(
          {ip, op, (uint32_t)c, (uint32_t)(elems * element), (uint32_t)elems, kDecBitshuffle});
      plan->scratch |= elems * element > kDecBuf;
      ip += c;
      op += elems * element;
    }
    const size_t left = size % 8 * element;
    if (left) {
      if (n - ip < left)
        return bad_data("bitshuffle decompression failed with code -1");
      plan->blocks.push_back({ip, op, (uint32_t)left, (uint32_t)left, 0, kDecRaw});
    }
    return SF_OK;
  }
  if (!std::strcmp(algorithm, "lz4")) {
    // decompress.cc:43-71, with block > 0 ? block : expected (:126-128).
    plan->algorithm = kChunkLz4;
    const size_t bsize = block > 0 ? block : expected;
    size_t read = 0, written = 0;
    while (written < expected) {
      if (read + 4 > n)
        return bad_data("lz4 data truncated");
      const size_t c = be32(p + read);
      read += 4;
      if (c == 0 || read + c > n)
        return bad_data("lz4 block size out of range");
      const size_t want = std::min(expected - written, bsize);
      if (want > 0xFFFFFFFFull || c >= kDecMaxIn) {
        t_last_error = "lz4 blocks of 4 GB or more (2 GB compressed) are not decoded on the "
                       "device";
        return SF_EUNSUPPORTED;
      }
      plan->blocks.push_back({read, written, (uint32_t)c, (uint32_t)want, 0, kDecLz4});
      read += c;
      written += want;
    }
    return SF_OK;
  }
  std::snprintf(text, sizeof text, "unknown compression algorithm %s", algorithm);
  return bad_data(text);
}

cudaError_t launch_decode(const uint8_t *d_payload, const DecodeBlock *d_blocks, size_t nblocks,
                          unsigned element, uint8_t *d_frame, uint8_t *d_scratch,
                          uint32_t *d_status, uint32_t *d_next, cudaStream_t stream) {
  if (nblocks == 0)
    return cudaSuccess;
  // One wave: the shared buffers allow 6 blocks of 4 warps an SM.
  const size_t want = (nblocks + kDecWarps - 1) / kDecWarps;
  const int grid = (int)std::min<size_t>(want, (size_t)device_sms() * 6);
  if (element == 2)
    k_decode<2><<<grid, kDecWarps * 32, 0, stream>>>(d_payload, d_blocks, (uint32_t)nblocks,
                                                     d_frame, d_scratch, d_status, d_next);
  else
    k_decode<4><<<grid, kDecWarps * 32, 0, stream>>>(d_payload, d_blocks, (uint32_t)nblocks,
                                                     d_frame, d_scratch, d_status, d_next);
  return cudaGetLastError();
}

std::string decode_error_text(const ChunkPlan &plan, const uint32_t status[3]) {
  char text[256];
  const int code = (int)(int32_t)status[2];
  if (plan.algorithm == kChunkBitshuffle)
    std::snprintf(text, sizeof text, "bitshuffle decompression failed with code %d", code);
  else if (status[0] == kDecShort)
    // The reference carries on from a short block; this decoder places
    // every block at its full size and refuses a chunk that does not fill it.
    std::snprintf(text, sizeof text, "lz4 block %u decompressed to %d bytes, expected %u",
                  status[1], code,
                  status[1] < plan.blocks.size() ? plan.blocks[status[1]].out_bytes : 0u);
  else
    std::snprintf(text, sizeof text, "lz4 decompression failed with code %d", code);
  return text;
}

}  // namespace sf
