// Whole-frame passes around the threshold:
//
//   k_scan<T>  mxi_max's scan<T> (apps/mxi_max.cc:47-67): the largest value
//              that is not a marker (max() - 1 a bad pixel, max() a tile
//              join), how many pixels are each marker, and how many valid
//              pixels are at 0xFFFD or above (the first 16-bit marker).
//   k_narrow   find_spots.cc:169-182, the --gpu-force narrowing of a 32-bit
//              frame to 16 bits: each value truncated to its low 16 bits (the
//              32-bit markers become the 16-bit ones) and the largest
//              non-marker value, which must be below 0xFFFD.
//
// Both read the frame once with 16-byte loads, four in flight a thread (a
// grid-stride loop over one wave of blocks), reduce within each warp and
// combine with one atomic per warp: HBM-bound passes.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "sf_frames.cuh"
#include "sf_stream.cuh"

namespace sf {
namespace {

constexpr int kScanThreads = 256;
constexpr int kLoads = 4;

template <typename T> struct Marks;
template <> struct Marks<uint16_t> {
  static constexpr uint32_t kJoin = 0xFFFFu, kDead = 0xFFFEu;
};
template <> struct Marks<uint32_t> {
  static constexpr uint32_t kJoin = 0xFFFFFFFFu, kDead = 0xFFFFFFFEu;
};

struct ScanAcc {
  uint32_t best = 0, dead = 0, join = 0, over = 0;
  template <typename T> __device__ __forceinline__ void add(uint32_t v) {
    dead += v == Marks<T>::kDead;
    join += v == Marks<T>::kJoin;
    const uint32_t real = v >= Marks<T>::kDead ? 0u : v;
    over += real >= 0xFFFDu;
    best = max(best, real);
  }
};

template <typename T>
__global__ void __launch_bounds__(kScanThreads)
k_scan(const T *__restrict__ img, size_t n, bool vec, unsigned long long *__restrict__ out) {
  ScanAcc a;
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  constexpr int kPer = 16 / sizeof(T);
  size_t done = 0;
  if (vec) {
    const uint4 *v4 = reinterpret_cast<const uint4 *>(img);
    const size_t nv = n / kPer;
    // kLoads loads in flight a thread before any is used.
    for (size_t i = tid; i < nv; i += kLoads * stride) {
      uint4 x[kLoads];
#pragma unroll
      for (int u = 0; u < kLoads; u++)
        x[u] = i + u * stride < nv ? __ldg(v4 + i + u * stride) : make_uint4(0, 0, 0, 0);
#pragma unroll
      for (int u = 0; u < kLoads; u++) {
        if (i + u * stride >= nv)
          break;
        const uint32_t w[4] = {x[u].x, x[u].y, x[u].z, x[u].w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
          if (sizeof(T) == 2) {
            a.add<T>(w[k] & 0xFFFFu);
            a.add<T>(w[k] >> 16);
          } else {
            a.add<T>(w[k]);
          }
        }
      }
    }
    done = nv * kPer;
  }
  for (size_t i = done + tid; i < n; i += stride)
    a.add<T>(img[i]);
  const uint32_t best = __reduce_max_sync(~0u, a.best);
  const uint32_t dead = __reduce_add_sync(~0u, a.dead);
  const uint32_t join = __reduce_add_sync(~0u, a.join);
  const uint32_t over = __reduce_add_sync(~0u, a.over);
  if ((threadIdx.x & 31) == 0) {
    if (best)
      atomicMax(out, (unsigned long long)best);
    if (dead)
      atomicAdd(out + 1, (unsigned long long)dead);
    if (join)
      atomicAdd(out + 2, (unsigned long long)join);
    if (over)
      atomicAdd(out + 3, (unsigned long long)over);
  }
}

__device__ __forceinline__ uint32_t narrow_real(uint32_t v) {
  return v >= 0xFFFFFFFEu ? 0u : v;
}

__global__ void __launch_bounds__(kScanThreads)
k_narrow(const uint32_t *__restrict__ in, size_t n, bool vec, uint16_t *__restrict__ out,
         uint32_t *__restrict__ worst) {
  uint32_t best = 0;
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t done = 0;
  if (vec) {
    const uint4 *v4 = reinterpret_cast<const uint4 *>(in);
    uint2 *o2 = reinterpret_cast<uint2 *>(out);
    const size_t nv = n / 4;
    for (size_t i = tid; i < nv; i += kLoads * stride) {
      uint4 x[kLoads];
#pragma unroll
      for (int u = 0; u < kLoads; u++)
        x[u] = i + u * stride < nv ? __ldg(v4 + i + u * stride) : make_uint4(0, 0, 0, 0);
#pragma unroll
      for (int u = 0; u < kLoads; u++) {
        if (i + u * stride >= nv)
          break;
        best = max(max(max(best, narrow_real(x[u].x)), narrow_real(x[u].y)),
                   max(narrow_real(x[u].z), narrow_real(x[u].w)));
        o2[i + u * stride] =
            make_uint2(__byte_perm(x[u].x, x[u].y, 0x5410), __byte_perm(x[u].z, x[u].w, 0x5410));
      }
    }
    done = nv * 4;
  }
  for (size_t i = done + tid; i < n; i += stride) {
    const uint32_t v = in[i];
    best = max(best, narrow_real(v));
    out[i] = (uint16_t)v;
  }
  best = __reduce_max_sync(~0u, best);
  if ((threadIdx.x & 31) == 0 && best)
    atomicMax(worst, best);
}

// One wave: 56 registers a thread leave room for 4 blocks of 256 an SM.
int scan_grid() { return device_sms() * 4; }

}  // namespace

cudaError_t launch_scan(const void *d_image, size_t n, unsigned bit_depth,
                        unsigned long long *d_out, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(d_out, 0, 4 * sizeof(unsigned long long), stream);
  if (e != cudaSuccess || n == 0)
    return e;
  const bool vec = reinterpret_cast<uintptr_t>(d_image) % 16 == 0;
  if (bit_depth == 16)
    k_scan<uint16_t><<<scan_grid(), kScanThreads, 0, stream>>>(
        static_cast<const uint16_t *>(d_image), n, vec, d_out);
  else
    k_scan<uint32_t><<<scan_grid(), kScanThreads, 0, stream>>>(
        static_cast<const uint32_t *>(d_image), n, vec, d_out);
  return cudaGetLastError();
}

cudaError_t launch_narrow(const uint32_t *d_in, size_t n, uint16_t *d_out, uint32_t *d_worst,
                          cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(d_worst, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess || n == 0)
    return e;
  const bool vec = reinterpret_cast<uintptr_t>(d_in) % 16 == 0 &&
                   reinterpret_cast<uintptr_t>(d_out) % 8 == 0;
  k_narrow<<<scan_grid(), kScanThreads, 0, stream>>>(d_in, n, vec, d_out, d_worst);
  return cudaGetLastError();
}

}  // namespace sf
