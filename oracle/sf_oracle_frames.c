/*
 * CPU oracle for the per-frame scans around the threshold. TEST
 * INFRASTRUCTURE ONLY: the checker for sf_scan_* and the narrowed threshold;
 * the product never links it.
 *
 *  - or_scan_u16 / or_scan_u32: mxi_max's scan<T> (apps/mxi_max.cc:47-67):
 *    the largest value that is not a marker (max() - 1 a bad pixel, max() a
 *    tile join), how many pixels are each marker, and how many valid pixels
 *    are at 0xFFFD or above.
 *  - or_narrow_to_16: find_spots.cc:169-182, the --gpu-force narrowing of a
 *    32-bit frame to 16 bits: every value truncated to its low 16 bits (the
 *    markers become the 16-bit markers), the largest non-marker value
 *    returned, and 1 if it is below 0xFFFD.
 */
#include <stddef.h>
#include <stdint.h>

#include "sf_oracle.h"

#define OR_SCAN(NAME, T, TOP)                                                        \
  void NAME(const T *pixels, size_t n, uint64_t out[4]) {                            \
    const T join = (T)(TOP), dead = (T)((TOP)-1u);                                   \
    T best = 0;                                                                      \
    uint64_t dead_n = 0, join_n = 0, above = 0;                                      \
    for (size_t i = 0; i < n; ++i) {                                                 \
      const T v = pixels[i];                                                         \
      dead_n += v == dead;                                                           \
      join_n += v == join;                                                           \
      const T real = v >= dead ? (T)0 : v;                                           \
      above += (uint64_t)real >= 0xFFFDu;                                            \
      best = real > best ? real : best;                                              \
    }                                                                                \
    out[0] = best;                                                                   \
    out[1] = dead_n;                                                                 \
    out[2] = join_n;                                                                 \
    out[3] = above;                                                                  \
  }

OR_SCAN(or_scan_u16, uint16_t, 0xFFFFu)
OR_SCAN(or_scan_u32, uint32_t, 0xFFFFFFFFu)

int or_narrow_to_16(const uint32_t *in, size_t n, uint16_t *out, uint32_t *offending) {
  uint32_t worst = 0;
  for (size_t i = 0; i < n; ++i) {
    const uint32_t v = in[i];
    const int marker = v >= 0xFFFFFFFEu;
    const uint32_t real = marker ? 0u : v;
    worst = real > worst ? real : worst;
    out[i] = (uint16_t)v;
  }
  *offending = worst;
  return worst < 0xFFFDu;
}
