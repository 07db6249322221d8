/*
 * Compressed chunks of synthetic frames, as a detector's HDF5 writer stores
 * them: the 12-byte filter header (uncompressed bytes as 8 big-endian bytes,
 * block bytes as 4) and then
 *
 *   bslz4  bitshuffle's blocks: per block of B elements (the last partial
 *          block rounded down to a multiple of 8) a 4-byte big-endian length
 *          and an LZ4 block of the block's bit planes (plane 8j + k holds
 *          bit k of byte j of every element, element i at bit i % 8 of the
 *          plane's byte i / 8); the size % 8 elements left over follow raw;
 *   lz4    blocks of the header's block bytes, each a 4-byte big-endian
 *          length and an LZ4 block.
 *
 * The LZ4 blocks are written by a greedy single-probe matcher (a 4096-entry
 * table of 4-byte prefixes) that keeps LZ4's end-of-block rules: no match
 * starts in the last 12 bytes of a block and the last 5 bytes are literals.
 * Blocks compress in parallel (OpenMP). These chunks stand in for detector
 * data in the tests and benchmarks of the device decoder.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "synth.h"

static void put_be32(uint8_t *p, uint32_t v) {
  p[0] = (uint8_t)(v >> 24), p[1] = (uint8_t)(v >> 16), p[2] = (uint8_t)(v >> 8),
  p[3] = (uint8_t)v;
}

static uint32_t read32(const uint8_t *p) {
  return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}

static size_t put_length(uint8_t *o, size_t v) {
  size_t n = 0;
  while (v >= 255) {
    o[n++] = 255;
    v -= 255;
  }
  o[n++] = (uint8_t)v;
  return n;
}

size_t sf_lz4_bound(size_t n) { return n + n / 255 + 16; }

/* One LZ4 block of src[0 .. n) into dst (at least sf_lz4_bound(n) bytes);
 * returns its length. */
size_t sf_lz4_block(const uint8_t *src, size_t n, uint8_t *dst) {
  enum { kHashBits = 12 };
  uint32_t table[1 << kHashBits];
  memset(table, 0, sizeof table);
  size_t ip = 0, anchor = 0, op = 0;
  if (n >= 13) {
    const size_t last_start = n - 12; /* a match starts at or before this */
    const size_t match_end = n - 5;   /* and ends at or before this */
    while (ip <= last_start) {
      const uint32_t v = read32(src + ip);
      const uint32_t h = (v * 2654435761u) >> (32 - kHashBits);
      const size_t cand = table[h];
      table[h] = (uint32_t)(ip + 1);
      if (cand == 0 || ip - (cand - 1) > 65535 || read32(src + cand - 1) != v) {
        ip++;
        continue;
      }
      const size_t from = cand - 1;
      size_t m = 4;
      while (ip + m < match_end && src[from + m] == src[ip + m])
        m++;
      const size_t lit = ip - anchor;
      uint8_t *token = dst + op++;
      *token = (uint8_t)((lit >= 15 ? 15 : lit) << 4 | (m - 4 >= 15 ? 15 : m - 4));
      if (lit >= 15)
        op += put_length(dst + op, lit - 15);
      memcpy(dst + op, src + anchor, lit);
      op += lit;
      const size_t off = ip - from;
      dst[op++] = (uint8_t)off;
      dst[op++] = (uint8_t)(off >> 8);
      if (m - 4 >= 15)
        op += put_length(dst + op, m - 4 - 15);
      ip += m;
      anchor = ip;
    }
  }
  const size_t lit = n - anchor;
  dst[op++] = (uint8_t)((lit >= 15 ? 15 : lit) << 4);
  if (lit >= 15)
    op += put_length(dst + op, lit - 15);
  memcpy(dst + op, src + anchor, lit);
  return op + lit;
}

/* The bit planes of n elements (n a multiple of 8) of esize bytes. */
void sf_bitshuffle(const uint8_t *in, uint8_t *out, size_t n, size_t esize) {
  const size_t row = n / 8;
  for (size_t j = 0; j < esize; j++)
    for (unsigned k = 0; k < 8; k++) {
      uint8_t *plane = out + (8 * j + k) * row;
      for (size_t g = 0; g < row; g++) {
        unsigned b = 0;
        for (unsigned t = 0; t < 8; t++)
          b |= ((in[(8 * g + t) * esize + j] >> k) & 1u) << t;
        plane[g] = (uint8_t)b;
      }
    }
}

static void header(uint8_t *out, size_t bytes, size_t block_bytes) {
  for (int i = 0; i < 8; i++)
    out[i] = (uint8_t)((uint64_t)bytes >> (56 - 8 * i));
  put_be32(out + 8, (uint32_t)block_bytes);
}

size_t sf_chunk_bound(size_t frame_bytes, size_t block_bytes) {
  const size_t b = block_bytes ? block_bytes : 8192;
  const size_t blocks = frame_bytes / b + 2;
  return 12 + frame_bytes + blocks * (4 + b / 255 + 16) + 64;
}

/* Blocks [0, nblocks) of `frame` compressed one by one into per-block
 * buffers, then laid out in order. */
static int64_t write_blocks(const uint8_t *frame, size_t nblocks, size_t block_bytes,
                            size_t last_bytes, size_t esize, int shuffle, uint8_t *out,
                            size_t cap, size_t at) {
  const size_t stride = 4 + sf_lz4_bound(block_bytes);
  uint8_t *tmp = malloc(nblocks * stride + 1);
  size_t *len = malloc((nblocks + 1) * sizeof(size_t));
  if (!tmp || !len) {
    free(tmp);
    free(len);
    return -1;
  }
  int bad = 0;
#pragma omp parallel
  {
    uint8_t *planes = shuffle ? malloc(block_bytes) : NULL;
    if (shuffle && !planes)
      bad = 1;
#pragma omp for schedule(dynamic, 16)
    for (long b = 0; b < (long)nblocks; b++) {
      if (shuffle && !planes)
        continue;
      const size_t bytes = (size_t)b + 1 == nblocks ? last_bytes : block_bytes;
      const uint8_t *src = frame + (size_t)b * block_bytes;
      if (shuffle) {
        sf_bitshuffle(src, planes, bytes / esize, esize);
        src = planes;
      }
      const size_t c = sf_lz4_block(src, bytes, tmp + (size_t)b * stride + 4);
      put_be32(tmp + (size_t)b * stride, (uint32_t)c);
      len[b] = c + 4;
    }
    free(planes);
  }
  if (bad) {
    free(tmp);
    free(len);
    return -1;
  }
  for (size_t b = 0; b < nblocks; b++) {
    if (at + len[b] > cap) {
      free(tmp);
      free(len);
      return -1;
    }
    memcpy(out + at, tmp + b * stride, len[b]);
    at += len[b];
  }
  free(tmp);
  free(len);
  return (int64_t)at;
}

int64_t sf_chunk_bslz4(const void *frame, size_t n_elems, unsigned esize, size_t block_bytes,
                       uint8_t *out, size_t cap) {
  if (!frame || !out || esize == 0 || cap < 12)
    return -1;
  /* bitshuffle's default block: 8192 bytes' worth, a multiple of 8, at
   * least 128 elements. */
  size_t block = block_bytes ? block_bytes / esize : 8192 / esize / 8 * 8;
  if (!block_bytes && block < 128)
    block = 128;
  if (block == 0 || block % 8)
    return -1;
  const uint8_t *src = frame;
  header(out, n_elems * esize, block * esize);
  const size_t nfull = n_elems / block;
  size_t last = n_elems % block;
  last -= last % 8;
  const size_t nblocks = nfull + (last ? 1 : 0);
  int64_t at = 12;
  if (nblocks) {
    at = write_blocks(src, nblocks, block * esize, (last ? last : block) * esize, esize, 1,
                      out, cap, 12);
    if (at < 0)
      return -1;
  }
  const size_t left = n_elems % 8 * esize;
  if ((size_t)at + left > cap)
    return -1;
  memcpy(out + at, src + (nfull * block + last) * esize, left);
  return at + (int64_t)left;
}

int64_t sf_chunk_lz4(const void *frame, size_t nbytes, size_t block_bytes, uint8_t *out,
                     size_t cap) {
  if (!frame || !out || cap < 12)
    return -1;
  const size_t block = block_bytes ? block_bytes : nbytes;
  header(out, nbytes, block_bytes);
  if (nbytes == 0)
    return 12;
  const size_t nblocks = (nbytes + block - 1) / block;
  const size_t last = nbytes - (nblocks - 1) * block;
  return write_blocks(frame, nblocks, block, last, 1, 0, out, cap, 12);
}
