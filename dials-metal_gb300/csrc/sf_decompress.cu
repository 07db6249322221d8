// Frame decompression on the device (sf_decompress.cuh).
//
// k_decode gives each block of a chunk to one warp:
//
//   LZ4     every lane follows the same parse of the block (its token, length
//           and offset bytes are the same loads for the whole warp); the
//           literal runs and matches are copied by the lanes together, 32
//           bytes apart. A match whose offset is shorter than its length
//           repeats a pattern of `offset` bytes: it is copied in passes of
//           D bytes from D bytes back, D doubling from the offset up to 128,
//           so that no pass reads what it writes.
//   planes  a bitshuffle block decodes into the warp's 8 KB of shared memory
//           (bitshuffle's default block is 8192 bytes); a lane then takes 8
//           elements at a time: for each byte j of an element, the byte of
//           each of the 8 planes 8j .. 8j + 7 at the group's column forms an
//           8 x 8 bit matrix whose transpose holds byte j of the 8 elements.
//           Larger blocks decode into a frame-sized scratch buffer instead.
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

__device__ __forceinline__ void prefetch_l1(const void *p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// One LZ4 block in[0, n) into dst[0, cap) by the whole warp. Returns the
// bytes produced, or minus (the input position where the stream was found
// bad) minus 1. The checks are LZ4_decompress_safe's: a literal run that
// reaches the last 12 bytes of output or the last 8 of input must end the
// block at the input's end; a match must start inside the output and end
// before its last 5 bytes.
template <typename Out>
__device__ __forceinline__ long long lz4_warp(const uint8_t *__restrict__ in, uint32_t n,
                                              Out *dst, uint32_t cap, int lane) {
  uint32_t ip = 0, op = 0;
  for (;;) {
    if (ip >= n)
      return -(long long)ip - 1;
    const uint32_t token = __ldg(in + ip++);
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
    // Passes of m <= D bytes from D back; D = off * 2^k while below 128.
    uint32_t D = off, done = 0;
    while (done < ml) {
      const uint32_t m = min(ml - done, min(D, 128u));
      Out *to = dst + op + done;
      for (uint32_t i = lane; i < m; i += 32)
        to[i] = to[(int)i - (int)D];
      __syncwarp();
      done += m;
      if (m == D && D < 128)
        D *= 2;
    }
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
         uint32_t *__restrict__ status) {
  __shared__ __align__(16) uint8_t buf[kDecWarps][kDecBuf];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t b = blockIdx.x * kDecWarps + warp; b < nblocks; b += gridDim.x * kDecWarps) {
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
      const long long r = lz4_warp(src, d.in_bytes, dst, d.out_bytes, lane);
      if (r < 0)
        report(status, kDecBad, b, r, lane);
      else if (r != (long long)d.out_bytes)
        report(status, kDecShort, b, r, lane);
      continue;
    }
    long long r;
    if (d.out_bytes <= kDecBuf) {
      r = lz4_warp(src, d.in_bytes, buf[warp], d.out_bytes, lane);
      if (r == (long long)d.out_bytes)
        unshuffle<E>(buf[warp], d.elems, dst, lane);
    } else {
      uint8_t *tmp = scratch + d.out_off;
      r = lz4_warp(src, d.in_bytes, tmp, d.out_bytes, lane);
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
      if (elems * element > 0xFFFFFFFFull) {
        t_last_error = "bitshuffle blocks of 4 GB or more are not decoded on the device";
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
      if (want > 0xFFFFFFFFull) {
        t_last_error = "lz4 blocks of 4 GB or more are not decoded on the device";
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
                          uint32_t *d_status, cudaStream_t stream) {
  if (nblocks == 0)
    return cudaSuccess;
  const size_t want = (nblocks + kDecWarps - 1) / kDecWarps;
  const int grid = (int)std::min<size_t>(want, (size_t)device_sms() * 16);
  if (element == 2)
    k_decode<2><<<grid, kDecWarps * 32, 0, stream>>>(d_payload, d_blocks, (uint32_t)nblocks,
                                                     d_frame, d_scratch, d_status);
  else
    k_decode<4><<<grid, kDecWarps * 32, 0, stream>>>(d_payload, d_blocks, (uint32_t)nblocks,
                                                     d_frame, d_scratch, d_status);
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
