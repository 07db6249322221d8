// Device-wide exclusive scan of uint32 values whose count lives on the
// device, so a pipeline of kernels never has to read a size back to the host.
// Two launches on a fixed grid: per-block chunk sums, then each block rescans
// its chunk with its offset, which it takes from its own block scan of the
// chunk sums (block 0 also writes the total). A thread takes kScanItems
// consecutive values (two 16-byte loads where the chunk allows), so a block
// scans kScanThreads * kScanItems values a step.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sf {

constexpr int kScanBlocks = 512;
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr uint32_t kScanStep = kScanThreads * kScanItems;  // values a block step
static_assert(kScanBlocks <= kScanThreads, "a chunk sum a thread in the offset scan");

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total (all threads see it).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
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
    const uint32_t w = lane < nwarps ? s_warp[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o)
        wi += t;
    }
    if (lane < nwarps)
      s_warp[lane] = wi - w;
    if (lane == 31)
      s_total = wi;
  }
  __syncthreads();
  const uint32_t r = s_warp[warp] + incl - v;
  *total = s_total;
  __syncthreads();
  return r;
}

// This block's share [lo, hi) of n values, in whole steps (so a share starts
// 16-byte aligned when the array does).
__device__ __forceinline__ void scan_chunk(uint32_t n, uint32_t *lo, uint32_t *hi) {
  const uint32_t per = (n + gridDim.x - 1) / gridDim.x;
  const uint32_t chunk = (per + kScanStep - 1) / kScanStep * kScanStep;
  *lo = (uint32_t)min((unsigned long long)n, (unsigned long long)blockIdx.x * chunk);
  *hi = (uint32_t)min((unsigned long long)n, (unsigned long long)*lo + chunk);
}

// A thread's kScanItems values from i (zero past hi).
__device__ __forceinline__ void scan_load(const uint32_t *__restrict__ in, uint32_t i,
                                          uint32_t hi, bool vec, uint32_t v[kScanItems]) {
  if (vec && i + kScanItems <= hi) {
    const uint4 a = *reinterpret_cast<const uint4 *>(in + i);
    const uint4 b = *reinterpret_cast<const uint4 *>(in + i + 4);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w;
    v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
    return;
  }
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
    v[k] = i + k < hi ? in[i + k] : 0u;
}
static_assert(kScanItems == 8, "two 16-byte loads a thread");

static __global__ void __launch_bounds__(kScanThreads)
scan_sums(const uint32_t *__restrict__ in, const uint32_t *__restrict__ d_n,
          uint32_t *__restrict__ block_sums, const uint32_t *__restrict__ d_error) {
  if (d_error && *d_error)
    return;
  uint32_t lo, hi;
  scan_chunk(*d_n, &lo, &hi);
  const bool vec = reinterpret_cast<uintptr_t>(in) % 16 == 0;
  uint32_t acc = 0;
  for (uint32_t i = lo + threadIdx.x * kScanItems; i < hi; i += kScanStep) {
    uint32_t v[kScanItems];
    scan_load(in, i, hi, vec, v);
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
      acc += v[k];
  }
  for (int o = 16; o; o >>= 1)
    acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ uint32_t s[32];
  if ((threadIdx.x & 31) == 0)
    s[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++)
      t += s[w];
    block_sums[blockIdx.x] = t;
  }
}

static __global__ void __launch_bounds__(kScanThreads)
scan_apply(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
           const uint32_t *__restrict__ d_n, const uint32_t *__restrict__ block_sums,
           uint32_t *__restrict__ d_total, const uint32_t *__restrict__ d_error) {
  if (d_error && *d_error)
    return;
  // This block's offset: the chunk sums of the blocks before it.
  __shared__ uint32_t s_carry;
  uint32_t all;
  const uint32_t bs = threadIdx.x < kScanBlocks ? block_sums[threadIdx.x] : 0u;
  const uint32_t be = block_exclusive_scan(bs, &all);
  if (threadIdx.x == blockIdx.x)
    s_carry = be;
  if (blockIdx.x == 0 && threadIdx.x == 0 && d_total)
    *d_total = all;
  __syncthreads();
  uint32_t lo, hi;
  scan_chunk(*d_n, &lo, &hi);
  const bool vec = reinterpret_cast<uintptr_t>(in) % 16 == 0 &&
                   reinterpret_cast<uintptr_t>(out) % 16 == 0;
  uint32_t carry = s_carry;
  for (uint32_t base = lo; base < hi; base += kScanStep) {  // block-uniform
    const uint32_t i = base + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    scan_load(in, i, hi, vec, v);  // all read before any is written (in may be out)
    uint32_t t = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
      const uint32_t x = v[k];
      v[k] = t;
      t += x;
    }
    uint32_t total;
    const uint32_t e = carry + block_exclusive_scan(t, &total);
    if (vec && i + kScanItems <= hi) {
      *reinterpret_cast<uint4 *>(out + i) = make_uint4(e + v[0], e + v[1], e + v[2], e + v[3]);
      *reinterpret_cast<uint4 *>(out + i + 4) =
          make_uint4(e + v[4], e + v[5], e + v[6], e + v[7]);
    } else {
#pragma unroll
      for (int k = 0; k < kScanItems; k++)
        if (i + k < hi)
          out[i + k] = e + v[k];
    }
    carry += total;
  }
}

// out[i] = sum of in[0..i) for i < *d_n; *d_total = sum of all. `in` and
// `out` may alias; d_total may not be d_n (block 0 writes it while the others
// read d_n). block_sums holds kScanBlocks words. Skipped entirely when
// *d_error is non-zero (d_error may be null).
inline cudaError_t exclusive_scan(const uint32_t *in, uint32_t *out, const uint32_t *d_n,
                                  uint32_t *d_total, uint32_t *block_sums,
                                  const uint32_t *d_error, cudaStream_t stream) {
  scan_sums<<<kScanBlocks, kScanThreads, 0, stream>>>(in, d_n, block_sums, d_error);
  scan_apply<<<kScanBlocks, kScanThreads, 0, stream>>>(in, out, d_n, block_sums, d_total,
                                                       d_error);
  return cudaGetLastError();
}

} // namespace sf
