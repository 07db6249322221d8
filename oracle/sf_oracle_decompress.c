/*
 * CPU oracle for frame decompression. TEST INFRASTRUCTURE ONLY: the checker
 * for the device decoder (sf_decompress_image, sf_find_compressed); the
 * product never links it.
 *
 * A restatement of decompress::image (src/spots/decompress.cc:77-134) and of
 * the two third-party decoders it calls, whose sources are absent from the
 * reference tree (the bitshuffle submodule is empty, its pin unknown):
 *
 *  - LZ4's block format, as LZ4_decompress_safe reads it: sequences of a
 *    token (literal length in the high nibble, match length - 4 in the low),
 *    255-continued length bytes, the literals, a 2-byte little-endian match
 *    offset; the last sequence holds literals only. The end-of-block rules
 *    are enforced as LZ4 enforces them: a literal run that reaches the last
 *    12 bytes of output or the last 8 of input must end the block exactly at
 *    the input's end, and a match may not reach the last 5 bytes of output.
 *  - bitshuffle's bshuf_decompress_lz4 (github.com/kiyo-masui/bitshuffle):
 *    blocks of block_size elements (0 selects 8192 bytes' worth, a multiple
 *    of 8 and at least 128; the last partial block is rounded down to a
 *    multiple of 8), each a 4-byte big-endian compressed length and an LZ4
 *    block of the block's bit planes; the size % 8 elements left over follow
 *    raw. A block's bit planes: plane 8j + k holds bit k of byte j of every
 *    element, element i at bit i % 8 of the plane's byte i / 8.
 *
 * Error texts are the reference's. Where bitshuffle returns a code the
 * reference prints it: -81 for a block size that is not a multiple of 8,
 * -91 for a block that does not decompress to its size; a chunk whose block
 * framing runs past its end (which bitshuffle, given no input length, would
 * read past) is refused here with code -1.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sf_oracle.h"

/* LZ4_decompress_safe(in, out, n, cap): bytes produced, or a negative code
 * (minus the input position where the stream was found bad, minus 1). */
long or_lz4_decode(const uint8_t *in, size_t n, uint8_t *out, size_t cap) {
  size_t ip = 0, op = 0;
  for (;;) {
    if (ip >= n)
      return -(long)ip - 1;
    const unsigned token = in[ip++];
    size_t lit = token >> 4;
    if (lit == 15) {
      unsigned s;
      do {
        if (ip >= n)
          return -(long)ip - 1;
        s = in[ip++];
        lit += s;
      } while (s == 255);
    }
    if (op + lit + 12 > cap || ip + lit + 8 > n) {
      /* The last sequence: its literals end the input and fit the output. */
      if (ip + lit != n || op + lit > cap)
        return -(long)ip - 1;
      memcpy(out + op, in + ip, lit);
      return (long)(op + lit);
    }
    memcpy(out + op, in + ip, lit);
    ip += lit;
    op += lit;
    const size_t off = (size_t)in[ip] | (size_t)in[ip + 1] << 8;
    ip += 2;
    if (off == 0 || off > op)
      return -(long)ip - 1;
    size_t ml = token & 15u;
    if (ml == 15) {
      unsigned s;
      do {
        if (ip >= n)
          return -(long)ip - 1;
        s = in[ip++];
        if (ip + 5 > n)
          return -(long)ip - 1;
        ml += s;
      } while (s == 255);
    }
    ml += 4;
    if (op + ml + 5 > cap)
      return -(long)ip - 1;
    /* Byte by byte: an offset shorter than the match repeats its pattern. */
    for (size_t i = 0; i < ml; i++)
      out[op + i] = out[op - off + i];
    op += ml;
  }
}

/* Element i, byte j, bit k <- plane 8j + k, bit i (the inverse of the bit
 * transposition bitshuffle stores). n is a multiple of 8. */
void or_bitunshuffle(const uint8_t *in, uint8_t *out, size_t n, size_t esize) {
  const size_t row = n / 8;
  memset(out, 0, n * esize);
  for (size_t j = 0; j < esize; j++)
    for (unsigned k = 0; k < 8; k++) {
      const uint8_t *plane = in + (8 * j + k) * row;
      for (size_t g = 0; g < row; g++) {
        const unsigned b = plane[g];
        if (!b)
          continue;
        for (unsigned t = 0; t < 8; t++)
          out[(8 * g + t) * esize + j] |= (uint8_t)(((b >> t) & 1u) << k);
      }
    }
}

size_t or_bshuf_default_block(size_t esize) {
  size_t b = 8192 / esize;
  b = b / 8 * 8;
  return b < 128 ? 128 : b;
}

static uint32_t be32(const uint8_t *p) {
  return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3];
}

/* bshuf_decompress_lz4(in, out, size, esize, block_size) over an input of
 * n_in bytes: input bytes consumed, or a negative code. */
long or_bshuf_decompress_lz4(const uint8_t *in, size_t n_in, uint8_t *out, size_t size,
                             size_t esize, size_t block_size) {
  if (block_size == 0)
    block_size = or_bshuf_default_block(esize);
  if (block_size % 8)
    return -81;
  const size_t nfull = size / block_size;
  size_t last = size % block_size;
  last -= last % 8;
  uint8_t *tmp = malloc(block_size * esize ? block_size * esize : 1);
  if (!tmp)
    return -1;
  size_t ip = 0, op = 0;
  for (size_t b = 0; b < nfull + (last ? 1 : 0); b++) {
    const size_t bs = b < nfull ? block_size : last;
    if (n_in - ip < 4) {
      free(tmp);
      return -1;
    }
    const size_t c = be32(in + ip);
    ip += 4;
    if (c > n_in - ip) {
      free(tmp);
      return -1;
    }
    const long r = or_lz4_decode(in + ip, c, tmp, bs * esize);
    if (r != (long)(bs * esize)) {
      free(tmp);
      return -91;
    }
    or_bitunshuffle(tmp, out + op, bs, esize);
    ip += c;
    op += bs * esize;
  }
  free(tmp);
  const size_t left = size % 8 * esize;
  if (n_in - ip < left)
    return -1;
  memcpy(out + op, in + ip, left);
  return (long)(ip + left);
}

size_t or_frame_bytes(size_t height, size_t width, unsigned bit_depth) {
  return height * width * bit_depth / 8; /* decompress.cc:72-75 */
}

static int say(char *err, size_t cap, const char *text) {
  if (err && cap) {
    strncpy(err, text, cap - 1);
    err[cap - 1] = 0;
  }
  return -1;
}

/* decompress::image: 0, or -1 with the reference's exception text in err. */
int or_decompress_image(const uint8_t *data, size_t n, const char *algorithm,
                        unsigned bit_depth, size_t height, size_t width, uint8_t *out,
                        size_t out_bytes, char *err, size_t err_cap) {
  char buf[256];
  const size_t expected = or_frame_bytes(height, width, bit_depth);
  const size_t element = bit_depth / 8;
  if (element == 0 || out_bytes < expected)
    return say(err, err_cap, "output buffer too small for the frame");
  if (!algorithm || !algorithm[0]) {
    if (n != expected) {
      snprintf(buf, sizeof buf, "uncompressed frame is %zu bytes, expected %zu", n, expected);
      return say(err, err_cap, buf);
    }
    memcpy(out, data, expected);
    return 0;
  }
  if (n < 12)
    return say(err, err_cap, "too short for a filter header");
  uint64_t usize = 0;
  for (int i = 0; i < 8; i++)
    usize = usize << 8 | data[i];
  const uint32_t block = be32(data + 8);
  if (usize != expected) {
    snprintf(buf, sizeof buf, "filter header says %llu bytes uncompressed, expected %zu",
             (unsigned long long)usize, expected);
    return say(err, err_cap, buf);
  }
  const uint8_t *payload = data + 12;
  const size_t pn = n - 12;
  if (!strcmp(algorithm, "bslz4")) {
    const long consumed = or_bshuf_decompress_lz4(payload, pn, out, expected / element, element,
                                                  block / element);
    if (consumed < 0) {
      snprintf(buf, sizeof buf, "bitshuffle decompression failed with code %ld", consumed);
      return say(err, err_cap, buf);
    }
    return 0;
  }
  if (!strcmp(algorithm, "lz4")) {
    /* decompress.cc:43-71 */
    const size_t bsize = block > 0 ? block : expected;
    size_t read = 0, written = 0;
    while (written < expected) {
      if (read + 4 > pn)
        return say(err, err_cap, "lz4 data truncated");
      const size_t c = be32(payload + read);
      read += 4;
      if (c == 0 || read + c > pn)
        return say(err, err_cap, "lz4 block size out of range");
      const size_t remaining = expected - written;
      const size_t want = remaining < bsize ? remaining : bsize;
      const long produced = or_lz4_decode(payload + read, c, out + written, want);
      if (produced < 0) {
        snprintf(buf, sizeof buf, "lz4 decompression failed with code %ld", produced);
        return say(err, err_cap, buf);
      }
      read += c;
      written += (size_t)produced;
    }
    return 0;
  }
  snprintf(buf, sizeof buf, "unknown compression algorithm %s", algorithm);
  return say(err, err_cap, buf);
}
