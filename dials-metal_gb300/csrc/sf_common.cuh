// Shared types and exact-decision helpers for the spot-finder kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sf_api.h"

namespace sf {

// Largest half-width the kernels are instantiated for (kernel_size 4,4); the
// stage-0 window then holds at most 9 x 9 = 81 pixels and the stage-2 window
// 13 x 13 = 169.
constexpr int kMaxHalf = 4;
constexpr int kMaxN0 = (2 * kMaxHalf + 1) * (2 * kMaxHalf + 1);

// Fixed-point scale of the sqrt(2 (n - 1)) bounds used by the integer
// stage-0 decision.
constexpr int kRootShift = 20;

// Per-launch constants, built on the host by make_launch_params().
struct LaunchParams {
  int algorithm;   // SF_DISPERSION_EXTENDED or SF_DISPERSION
  int half;        // kernel half-width (square windows)
  double gain, sigma_b, sigma_s;
  uint32_t min_local;
  uint64_t p_min;  // a candidate pixel needs value >= p_min (global threshold)
  int int_ok;      // gain == 1 and integral sigmas: the integer decisions hold
  uint32_t sigma_b_int, sigma_s2_int;
  // Indexed by the window count n (0 .. kMaxN0):
  uint32_t root_lo[kMaxN0 + 1], root_hi[kMaxN0 + 1]; // floor/ceil(r_n 2^20)
  double root[kMaxN0 + 1];  // r_n = RN(sqrt(2 (n - 1))), the reference's value
  float rootf[kMaxN0 + 1];  // RN_float(sqrtf(2 (n - 1))), for 16-bit frames
};

// Reference SignalPixel layout (src/spots/signal_pixel.hh:20-28).
static_assert(sizeof(sf_signal_pixel) == 16, "SignalPixel is 16 bytes");

// Pixel-type traits, mirroring src/spots/dext.hh:18-38: window sums in W,
// tests in R, masked at max - 1 and above.
template <typename T> struct Traits;
template <> struct Traits<uint32_t> {
  using W = unsigned long long;
  static constexpr uint32_t kMasked = 0xFFFFFFFEu;
  static constexpr uint32_t kOutside = 0xFFFFFFFFu;
};
template <> struct Traits<uint16_t> {
  using W = uint32_t;
  static constexpr uint32_t kMasked = 0xFFFEu;
  static constexpr uint32_t kOutside = 0xFFFFu;
};

// ---------------------------------------------------------------------------
// Stage 0, 32-bit frames: the dispersion test of src/spots/dext.cc:99-109,
//   ((m s2 - s s) - g s (m - 1)) > ((g s) sigma_b) sqrt(2 (m - 1))
// in double with every operation rounded separately.
//
// Integer route (gain 1, integral sigma_b): when Q < 2^46 and S < 2^26 every
// product and difference on the left is an integer below 2^53, so the double
// left side is exactly A = n Q - S^2 - S (n - 1). The right side is
// RN(X) with X = (S sigma_b) r_n, S sigma_b exact. With r_n bracketed by
// [lo, hi] / 2^20, X lies in [XL, XU]; A > RN(X) holds when XU <= A - 2 (then
// X < A - 1 and RN(X) <= A - 1) and fails when XL >= A (then RN(X) >= A).
// Anything between goes to the double sequence, which is the reference's.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool stage0_double(uint32_t n, unsigned long long S,
                                              unsigned long long Q,
                                              const LaunchParams &P) {
  const double m = (double)n;
  const double s = __ull2double_rn(S);
  const double s2 = __ull2double_rn(Q);
  const double gs = __dmul_rn(P.gain, s);
  const double m1 = __dsub_rn(m, 1.0);
  const double lhs = __dsub_rn(__dsub_rn(__dmul_rn(m, s2), __dmul_rn(s, s)),
                               __dmul_rn(gs, m1));
  const double rhs = __dmul_rn(__dmul_rn(gs, P.sigma_b), P.root[n]);
  return lhs > rhs;
}

__device__ __forceinline__ bool stage0_u32(uint32_t n, unsigned long long S,
                                           unsigned long long Q,
                                           const LaunchParams &P,
                                           const uint32_t *root_lo,
                                           const uint32_t *root_hi) {
  if (n < P.min_local)
    return false;
  if (n == 0)
    return false; // S = Q = 0: 0 > 0 * NaN is false in the reference too
  if (P.int_ok && S < (1ull << 26) && Q < (1ull << 46)) {
    const long long A = (long long)(n * Q) - (long long)(S * S) -
                        (long long)(S * (unsigned long long)(n - 1));
    const unsigned long long B = S * P.sigma_b_int; // < 2^36
    const long long XL = (long long)((B * root_lo[n]) >> kRootShift);
    const long long XU =
        (long long)((B * root_hi[n] + ((1ull << kRootShift) - 1)) >> kRootShift);
    if (XU <= A - 2)
      return true;
    if (XL >= A)
      return false;
  }
  return stage0_double(n, S, Q, P);
}

// ---------------------------------------------------------------------------
// Stage 2, 32-bit frames: src/spots/dext.cc:203-217 at a candidate pixel,
//   mean = n >= min_local ? S / n : 0;  p >= mean + sigma_s sqrt(g mean)
// and the emitted background float(mean).
//
// Integer route (gain 1, integral sigma_s, S < 2^24): with d = n p - S,
// d < 0 means p < mean by at least 1/n, far more than an ulp, so RN(mean)
// > p and the test fails. Otherwise E = d^2 - sigma_s^2 S n has the sign of
// p - t for t = mean + sigma_s sqrt(mean), and |E| > 8192 puts p further from
// t than the double sequence's rounding can move it (at most 2^-50 t with t <
// 2^24.4 and sigma_s <= 1024). Near ties go to the double sequence.
//
// float(RN_double(S / n)) equals RN_float(S / n) for these rationals: one
// that is not exactly a float midpoint is at least 2^-32 relative from every
// midpoint, far more than the 2^-53 a double rounding moves it. So the
// background is an IEEE float division, exact in its inputs for S < 2^24.
// ---------------------------------------------------------------------------
// The reference's double sequence (dext.cc:204-206), out of line: callers
// reach it rarely and should not issue it otherwise.
static __device__ __noinline__ bool stage2_double(uint32_t p, uint32_t n, unsigned long long S,
                                                  const LaunchParams &P, float *bg) {
  const double mean = __ddiv_rn(__ull2double_rn(S), (double)n);
  *bg = __double2float_rn(mean);
  const double t = __dadd_rn(mean, __dmul_rn(P.sigma_s, __dsqrt_rn(__dmul_rn(P.gain, mean))));
  return (double)p >= t;
}

__device__ __forceinline__ bool stage2_u32(uint32_t p, uint32_t n,
                                           unsigned long long S,
                                           const LaunchParams &P, float *bg) {
  if (n < P.min_local) {
    // mean 0: sqrt(gain 0) is a zero, sigma_s times it a zero (both finite),
    // and p >= 0 + 0 holds for every pixel.
    *bg = 0.0f;
    return true;
  }
  if (P.int_ok && S < (1ull << 24)) {
    *bg = __fdiv_rn((float)(uint32_t)S, (float)n);
    const long long d = (long long)n * (long long)p - (long long)S;
    if (d < 0)
      return false;
    if (d >= (1ll << 31))
      return true; // p - mean > 2^23.6 > sigma_s sqrt(mean) + any rounding
    const long long E =
        d * d - (long long)P.sigma_s2_int * (long long)S * (long long)n;
    // |p - t| beyond the double sequence's error err <= 2^-50 t means
    // |E| > n^2 err (err + 2 sigma_s sqrt(mean)); bound that from above in
    // float with generous slack (mean < 2^24 here).
    const float mu = __fdiv_ru((float)(uint32_t)S, (float)n);
    const float rt = __fsqrt_ru(mu) * 1.001f + 1.0f;
    const float ss = (float)P.sigma_s;
    const float t = mu + ss * rt + 1.0f;
    const float err = t * 0x1p-49f;
    const float nn = (float)n * (float)n;
    const float bound = nn * err * (err + 2.0f * ss * rt) * 2.0f + 1.0f;
    const float Ef = (float)E;
    if (Ef > bound)
      return true;
    if (Ef < -bound)
      return false;
  }
  return stage2_double(p, n, S, P, bg);
}

// ---------------------------------------------------------------------------
// 16-bit frames: the tests are float (src/spots/dext.hh:31-33) and cheap, so
// they run as the reference's sequence of IEEE float operations.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool stage0_u16(uint32_t n, uint32_t S, uint32_t Q,
                                           const LaunchParams &P) {
  if (n < P.min_local)
    return false;
  const float g = (float)P.gain, sb = (float)P.sigma_b;
  const float m = __uint2float_rn(n);
  const float s = __uint2float_rn(S);
  const float s2 = __uint2float_rn(Q);
  const float gs = __fmul_rn(g, s);
  const float lhs = __fsub_rn(__fsub_rn(__fmul_rn(m, s2), __fmul_rn(s, s)),
                              __fmul_rn(gs, __fsub_rn(m, 1.0f)));
  const float rhs = __fmul_rn(__fmul_rn(gs, sb), P.rootf[n]);
  return lhs > rhs;
}

__device__ __forceinline__ bool stage2_u16(uint32_t p, uint32_t n, uint32_t S,
                                           const LaunchParams &P, float *bg) {
  const float g = (float)P.gain, ss = (float)P.sigma_s;
  const float mean =
      n >= P.min_local ? __fdiv_rn(__uint2float_rn(S), __uint2float_rn(n)) : 0.0f;
  *bg = mean;
  return __uint2float_rn(p) >= __fadd_rn(mean, __fmul_rn(ss, __fsqrt_rn(__fmul_rn(g, mean))));
}

} // namespace sf
