// 3-D spot labelling on the device: the streaming grouping of
// src/spots/dials_spots.cc (Labeller::add / flush / emit / finish), for a
// batch of frames at a time.
//
// State carried between batches is the reference's: the "live" pixels of
// every component that still touches the newest frame, in (frame, index)
// order, each pointing straight at its component's first pixel
// (dials_spots.cc:199-218). A batch of B frames is appended to that pool in
// order and joined in one union-find pass -- left neighbour in the row,
// the pixel above, the same pixel on the previous frame when the frames are
// consecutive (dials_spots.cc:106-137) -- with every link toward the lower
// position, so a root is its component's first pixel (:36-55).
//
// What the reference emits at each flush is the components with no pixel on
// the frame just added, in order of first pixel (:162-194). Over a batch that
// is: every component whose last frame is not the batch's last frame, ordered
// by (last frame, first pixel), which a stable partition of the closing roots
// by last frame produces. Each emitted component's members are sorted back
// into (frame, index) order and the reference's emit() arithmetic runs over
// them sequentially in double, so the spot table is the reference's bit for
// bit (:221-360).

#include <cuda_runtime.h>
#include <stdint.h>

#include <climits>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "sf_api.h"
#include "sf_common.cuh"
#include "sf_label.cuh"
#include "sf_scan.cuh"

namespace sf {

extern thread_local std::string t_last_error;
int fail(cudaError_t e, const char *what);

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kThreads = 256;
constexpr int kGrid = 2 * 152;          // persistent grid-stride launches
constexpr int kWarpSortMax = 1024;      // members sorted by one warp
constexpr int kBlockSortMax = 8192;     // members sorted by one block
constexpr int kUnionRetries = 1 << 20;  // cap on a union's CAS retries

enum : uint32_t {
  kErrLiveFull = 1u,   // more open pixels than the live pool holds
  kErrUnion = 2u,      // a union did not settle within kUnionRetries
  kErrSpotSize = 4u,   // an accepted spot larger than kBlockSortMax
  kErrOutFull = 8u,    // more spots / kept pixels than the batch outputs hold
  kErrListOverflow = 16u, // an input list's count exceeds its stride
};

enum { kCntSignal = 0, kCntGroups, kCntSmall, kCntLarge, kCntSeparated, kCntAccepted };

struct LabelStatus {
  uint32_t error;
  uint32_t n_live;      // open pixels carried into the next batch
  uint32_t prev_start;  // first live position of the last added frame
  uint32_t n_total;     // n_live + the batch's pixels
  uint32_t n_closing, n_cand, n_cand_pixels, n_accept, n_accept_pixels, n_open;
  uint32_t frame_off[kLabelMaxBatch + 1];
  unsigned long long counts[6];
};

// One call's arguments. They live in device memory (copied in before every
// call) so that a captured launch sequence can be replayed with new ones.
struct BatchArgs {
  const sf_signal_pixel *lists;  // frame j's list at lists + j * stride
  const uint32_t *counts;        // frame j's count
  unsigned long long stride;
  unsigned long long pixel_base;  // kept pixels stored before this call
  int nb;
  int finishing;        // close everything (finish(), dials_spots.cc:147-151)
  int two_d;
  uint32_t width, npix;
  uint32_t min_size, max_size;
  double max_separation;
  int32_t frames[kLabelMaxBatch];
  uint8_t link_prev[kLabelMaxBatch];
};

// ---------------------------------------------------------------------------
// Union-find (dials_spots.cc:36-55), lock-free: a link is a CAS on a root
// toward the smaller position, and finds halve paths.
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t uf_find(uint32_t *parent, uint32_t x) {
  volatile uint32_t *vp = parent;
  while (true) {
    const uint32_t p = vp[x];
    if (p == x)
      return x;
    const uint32_t gp = vp[p];
    if (gp == p)
      return p;
    vp[x] = gp; // gp is an ancestor of x: a benign shortcut
    x = gp;
  }
}

__device__ __forceinline__ void uf_unite(uint32_t *parent, uint32_t a, uint32_t b,
                                         LabelStatus *st) {
  for (int it = 0; it < kUnionRetries; it++) {
    a = uf_find(parent, a);
    b = uf_find(parent, b);
    if (a == b)
      return;
    if (a < b) {
      const uint32_t t = a;
      a = b;
      b = t;
    }
    const uint32_t old = atomicCAS(&parent[a], a, b);
    if (old == a)
      return;
  }
  atomicOr(&st->error, kErrUnion);
}

__device__ __forceinline__ uint32_t lower_bound(const uint32_t *v, uint32_t lo, uint32_t hi,
                                                uint32_t key) {
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (v[mid] < key)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// Kernels of one batch, in launch order.
// ---------------------------------------------------------------------------

__global__ void k_offsets(LabelStatus *st, const BatchArgs *__restrict__ ap,
                          uint32_t capacity) {
  if (threadIdx.x != 0 || st->error)
    return;
  const BatchArgs &a = *ap;
  const uint32_t *counts = a.counts;
  const size_t stride = a.stride;
  uint32_t off = 0;
  for (int j = 0; j < a.nb; j++) {
    st->frame_off[j] = off;
    // A list whose count exceeds its stride is one that overflowed its
    // threshold's capacity: it is incomplete, and refused.
    if (counts[j] > stride) {
      st->error |= kErrListOverflow;
      return;
    }
    off += counts[j];
  }
  st->frame_off[a.nb] = off;
  const unsigned long long total = (unsigned long long)st->n_live + off;
  if (total > capacity) {
    st->error |= kErrLiveFull;
    return;
  }
  st->n_total = (uint32_t)total;
  st->counts[kCntSignal] += off;
}

__global__ void k_append(LabelStatus *st, const BatchArgs *__restrict__ ap, int32_t *frame,
                         uint32_t *index, uint32_t *value, uint32_t *parent) {
  if (st->error)
    return;
  const BatchArgs &a = *ap;
  const sf_signal_pixel *__restrict__ lists = a.lists;
  const size_t stride = a.stride;
  const int j = blockIdx.y;
  const uint32_t n = st->frame_off[j + 1] - st->frame_off[j];
  const uint32_t base = st->n_live + st->frame_off[j];
  const sf_signal_pixel *list = lists + (size_t)j * stride;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const sf_signal_pixel s = list[i];
    const uint32_t p = base + i;
    frame[p] = a.frames[j];
    index[p] = s.index;
    value[p] = s.value;
    parent[p] = p;
  }
}

// dials_spots.cc:106-137: left (same row), above (same frame), and the same
// index on the previous frame when it is the one before.
__global__ void k_link(LabelStatus *st, const BatchArgs *__restrict__ ap,
                       const uint32_t *__restrict__ index, uint32_t *parent) {
  const BatchArgs &a = *ap;
  if (st->error)
    return;
  const int j = blockIdx.y;
  const uint32_t width = a.width;
  const uint32_t start = st->n_live + st->frame_off[j];
  const uint32_t end = st->n_live + st->frame_off[j + 1];
  uint32_t plo = 0, phi = 0;
  if (a.link_prev[j]) {
    plo = j == 0 ? st->prev_start : st->n_live + st->frame_off[j - 1];
    phi = j == 0 ? st->n_live : start;
  }
  for (uint32_t p = start + blockIdx.x * blockDim.x + threadIdx.x; p < end;
       p += gridDim.x * blockDim.x) {
    const uint32_t idx = index[p];
    if (p > start && idx % width != 0 && index[p - 1] == idx - 1)
      uf_unite(parent, p, p - 1, st);
    if (idx >= width) {
      const uint32_t t = idx - width;
      const uint32_t q = lower_bound(index, start, p, t);
      if (q < p && index[q] == t)
        uf_unite(parent, p, q, st);
    }
    if (phi > plo) {
      const uint32_t q = lower_bound(index, plo, phi, idx);
      if (q < phi && index[q] == idx)
        uf_unite(parent, p, q, st);
    }
  }
}

__global__ void k_flatten(LabelStatus *st, uint32_t *parent, uint32_t *root, int32_t *zlast,
                          uint32_t *csize, uint32_t *candid) {
  if (st->error)
    return;
  const uint32_t n = st->n_total;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += gridDim.x * blockDim.x) {
    uint32_t r = p;
    while (parent[r] != r)
      r = parent[r];
    root[p] = r;
    zlast[p] = INT_MIN;
    csize[p] = 0;
    candid[p] = kNone;
  }
}

__global__ void k_comp_stats(LabelStatus *st, const uint32_t *__restrict__ root,
                             const int32_t *__restrict__ frame, int32_t *zlast,
                             uint32_t *csize) {
  if (st->error)
    return;
  const uint32_t n = st->n_total;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += gridDim.x * blockDim.x) {
    const uint32_t r = root[p];
    atomicMax(&zlast[r], frame[p]);
    atomicAdd(&csize[r], 1u);
  }
}

__device__ __forceinline__ bool closes(const BatchArgs &a, int32_t z) {
  return a.finishing || a.two_d || z < a.frames[a.nb - 1];
}

// Emission event of a component that closes: at finish() one flush; else the
// add() of the frame after its last one (dials_spots.cc:65-69, :144).
__device__ __forceinline__ uint32_t bucket_of(const BatchArgs &a, int32_t z) {
  if (a.finishing || z < a.frames[0])
    return 0;
  int lo = 0, hi = a.nb - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a.frames[mid] < z)
      lo = mid + 1;
    else
      hi = mid;
  }
  return 1u + (uint32_t)lo;
}

__global__ void k_closing_flags(LabelStatus *st, const BatchArgs *__restrict__ ap,
                                const uint32_t *__restrict__ root,
                                const int32_t *__restrict__ zlast, uint32_t *flag,
                                uint32_t *open) {
  const BatchArgs &a = *ap;
  if (st->error)
    return;
  const uint32_t n = st->n_total;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += gridDim.x * blockDim.x) {
    const uint32_t r = root[p];
    const bool c = closes(a, zlast[r]);
    flag[p] = (r == p && c) ? 1u : 0u;
    open[p] = c ? 0u : 1u;
  }
}

__global__ void k_closing_list(LabelStatus *st, const BatchArgs *__restrict__ ap,
                               const uint32_t *__restrict__ flag,
                               const uint32_t *__restrict__ pos,
                               const int32_t *__restrict__ zlast, uint32_t *clist,
                               uint32_t *cbucket) {
  const BatchArgs &a = *ap;
  if (st->error)
    return;
  const uint32_t n = st->n_total;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += gridDim.x * blockDim.x) {
    if (flag[p]) {
      const uint32_t k = pos[p];
      clist[k] = p;
      cbucket[k] = bucket_of(a, zlast[p]);
    }
  }
}

// Stable partition of the closing roots by emission event.
constexpr int kBuckets = kLabelMaxBatch + 1;

__global__ void __launch_bounds__(kThreads)
k_bucket_hist(LabelStatus *st, const uint32_t *__restrict__ cbucket, uint32_t *hist) {
  if (st->error)
    return;
  __shared__ uint32_t h[kBuckets];
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
    h[b] = 0;
  __syncthreads();
  uint32_t lo, hi;
  scan_chunk(st->n_closing, &lo, &hi);
  for (uint32_t k = lo + threadIdx.x; k < hi; k += blockDim.x)
    atomicAdd(&h[cbucket[k]], 1u);
  __syncthreads();
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
    hist[blockIdx.x * kBuckets + b] = h[b];
}

// Exclusive scan over (bucket, block) in bucket-major order, in place.
__global__ void __launch_bounds__(1024) k_bucket_offsets(LabelStatus *st, uint32_t *hist) {
  if (st->error)
    return;
  __shared__ uint32_t btotal[kBuckets];
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) {
    uint32_t run = 0;
    for (int blk = 0; blk < kGrid; blk++) {
      const uint32_t v = hist[blk * kBuckets + b];
      hist[blk * kBuckets + b] = run;
      run += v;
    }
    btotal[b] = run;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int b = 0; b < kBuckets; b++) {
      const uint32_t v = btotal[b];
      btotal[b] = run;
      run += v;
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
    for (int blk = 0; blk < kGrid; blk++)
      hist[blk * kBuckets + b] += btotal[b];
}

__global__ void __launch_bounds__(kThreads)
k_bucket_scatter(LabelStatus *st, const uint32_t *__restrict__ clist,
                 const uint32_t *__restrict__ cbucket, const uint32_t *__restrict__ hist,
                 uint32_t *order) {
  if (st->error)
    return;
  constexpr int W = kThreads / 32;
  __shared__ uint32_t wcnt[W][kBuckets];
  __shared__ uint32_t running[kBuckets];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
    running[b] = hist[blockIdx.x * kBuckets + b];
  uint32_t lo, hi;
  scan_chunk(st->n_closing, &lo, &hi);
  for (uint32_t base = lo; base < hi; base += blockDim.x) {
    for (int i = threadIdx.x; i < W * kBuckets; i += blockDim.x)
      (&wcnt[0][0])[i] = 0;
    __syncthreads();
    const uint32_t k = base + threadIdx.x;
    const bool valid = k < hi;
    const uint32_t b = valid ? cbucket[k] : kBuckets; // kBuckets: no bucket
    const unsigned m = __match_any_sync(0xffffffffu, b);
    const uint32_t rank = __popc(m & ((1u << lane) - 1u));
    if (valid && rank == 0)
      wcnt[warp][b] = __popc(m);
    __syncthreads();
    // Exclusive prefix over warps, per bucket; the running totals advance.
    for (int bb = threadIdx.x; bb < kBuckets; bb += blockDim.x) {
      uint32_t run = running[bb];
      for (int w = 0; w < W; w++) {
        const uint32_t v = wcnt[w][bb];
        wcnt[w][bb] = run;
        run += v;
      }
      running[bb] = run;
    }
    __syncthreads();
    if (valid)
      order[wcnt[warp][b] + rank] = clist[k];
    __syncthreads();
  }
}

// Size filters (dials_spots.cc:224-231) over the closing components in
// emission order.
__global__ void k_size_filter(LabelStatus *st, const BatchArgs *__restrict__ ap,
                              const uint32_t *__restrict__ order,
                              const uint32_t *__restrict__ csize, uint32_t *cflag) {
  const BatchArgs &a = *ap;
  if (st->error)
    return;
  const uint32_t n = st->n_closing;
  uint32_t small = 0, large = 0, groups = 0;
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += gridDim.x * blockDim.x) {
    const uint32_t sz = csize[order[e]];
    groups++;
    const bool s = sz < a.min_size, l = sz > a.max_size;
    small += s;
    large += !s && l;
    cflag[e] = (!s && !l) ? 1u : 0u;
  }
  for (int o = 16; o; o >>= 1) {
    small += __shfl_xor_sync(0xffffffffu, small, o);
    large += __shfl_xor_sync(0xffffffffu, large, o);
    groups += __shfl_xor_sync(0xffffffffu, groups, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (groups)
      atomicAdd(&st->counts[kCntGroups], (unsigned long long)groups);
    if (small)
      atomicAdd(&st->counts[kCntSmall], (unsigned long long)small);
    if (large)
      atomicAdd(&st->counts[kCntLarge], (unsigned long long)large);
  }
}

__global__ void k_cand_list(LabelStatus *st, const uint32_t *__restrict__ order,
                            const uint32_t *__restrict__ csize,
                            const uint32_t *__restrict__ cflag,
                            const uint32_t *__restrict__ cpos, uint32_t *cand_root,
                            uint32_t *cand_n, uint32_t *candid, uint32_t *cursor) {
  if (st->error)
    return;
  const uint32_t n = st->n_closing;
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += gridDim.x * blockDim.x) {
    if (cflag[e]) {
      const uint32_t c = cpos[e], r = order[e];
      cand_root[c] = r;
      cand_n[c] = csize[r];
      candid[r] = c;
      cursor[c] = 0;
    }
  }
}

__global__ void k_gather(LabelStatus *st, const uint32_t *__restrict__ root,
                         const uint32_t *__restrict__ candid,
                         const uint32_t *__restrict__ cand_off, uint32_t *cursor,
                         uint32_t *members) {
  if (st->error)
    return;
  const uint32_t n = st->n_total;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += gridDim.x * blockDim.x) {
    const uint32_t c = candid[root[p]];
    if (c != kNone) {
      const uint32_t slot = atomicAdd(&cursor[c], 1u);
      members[cand_off[c] + slot] = p;
    }
  }
}

// Bitonic sort of m values (padded to a power of two with kNone) in shared
// memory by `nt` cooperating threads numbered t.
__device__ void bitonic_sort(uint32_t *s, int m, int t, int nt, bool warp_only) {
  int size = 1;
  while (size < m)
    size <<= 1;
  for (int i = m + t; i < size; i += nt)
    s[i] = kNone;
  if (warp_only)
    __syncwarp();
  else
    __syncthreads();
  for (int k = 2; k <= size; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = t; i < size; i += nt) {
        const int l = i ^ j;
        if (l > i) {
          const uint32_t x = s[i], y = s[l];
          const bool up = (i & k) == 0;
          if ((x > y) == up) {
            s[i] = y;
            s[l] = x;
          }
        }
      }
      if (warp_only)
        __syncwarp();
      else
        __syncthreads();
    }
  }
}

// The first-pass sums of the reference's emit() (dials_spots.cc:240-276) in
// integers. Every term of its double accumulations is an integer (the value,
// its square) or a half-integer (the value times a pixel centre c + 0.5), so
// while each sum stays below 2^53 (2^52 for the half-integers) every partial
// sum is exact in double and the doubles equal these integers, whatever the
// order. W[ax] holds twice the weighted sum. `exact` is false when a bound
// could fail; the double sequence then runs instead.
struct FirstPass {
  unsigned long long S, Q2, W[3];
  int32_t bb[6];  // x0, x1, y0, y1, z0, z1
  // The brightest pixel, ties to the first in member order; none (all ones)
  // until a value above 0, where the reference's peak stays at (0, 0, 0).
  uint32_t peak_v, peak_k;
  bool exact;
};

__device__ __forceinline__ void fp_init(FirstPass &f) {
  f.S = f.Q2 = f.W[0] = f.W[1] = f.W[2] = 0;
  f.bb[0] = f.bb[2] = f.bb[4] = INT_MAX;
  f.bb[1] = f.bb[3] = f.bb[5] = INT_MIN;
  f.peak_v = 0;
  f.peak_k = 0xFFFFFFFFu;
  f.exact = true;
}

__device__ __forceinline__ void fp_add(FirstPass &f, uint32_t k, uint32_t v, int32_t x,
                                       int32_t y, int32_t z) {
  // v < 2^26 keeps v^2 < 2^52; coordinates below 2^20 keep v (2c + 1) < 2^53;
  // negative frames would make partial sums exceed the total.
  f.exact = f.exact && v < (1u << 26) && z >= 0 && x < (1 << 20) && y < (1 << 20) &&
            z < (1 << 20);
  const unsigned long long vv = v;
  f.S += vv;
  f.Q2 += vv * vv;
  f.W[0] += vv * (unsigned long long)(2 * x + 1);
  f.W[1] += vv * (unsigned long long)(2 * y + 1);
  f.W[2] += vv * (unsigned long long)(2 * (long long)z + 1);
  f.bb[0] = min(f.bb[0], x), f.bb[1] = max(f.bb[1], x + 1);
  f.bb[2] = min(f.bb[2], y), f.bb[3] = max(f.bb[3], y + 1);
  f.bb[4] = min(f.bb[4], z), f.bb[5] = max(f.bb[5], z + 1);
  if (v > 0 && (v > f.peak_v || (v == f.peak_v && k < f.peak_k))) {
    f.peak_v = v;
    f.peak_k = k;
  }
}

__device__ __forceinline__ void fp_merge(FirstPass &f, const FirstPass &g) {
  f.S += g.S;
  f.Q2 += g.Q2;
  for (int a = 0; a < 3; a++)
    f.W[a] += g.W[a];
  for (int a = 0; a < 6; a += 2) {
    f.bb[a] = min(f.bb[a], g.bb[a]);
    f.bb[a + 1] = max(f.bb[a + 1], g.bb[a + 1]);
  }
  if (g.peak_k != 0xFFFFFFFFu &&
      (g.peak_v > f.peak_v || (g.peak_v == f.peak_v && g.peak_k < f.peak_k))) {
    f.peak_v = g.peak_v;
    f.peak_k = g.peak_k;
  }
  f.exact = f.exact && g.exact;
}

__device__ __forceinline__ bool fp_finish(FirstPass &f) {
  const unsigned long long lim = 1ull << 53;
  f.exact = f.exact && f.S < lim && f.Q2 < lim && f.W[0] < lim && f.W[1] < lim && f.W[2] < lim;
  return f.exact;
}

// The member's pixel: (x, y, z) and value.
__device__ __forceinline__ void member(const uint32_t q, const int32_t *frame,
                                       const uint32_t *index, const uint32_t *value,
                                       uint32_t width, int32_t *x, int32_t *y, int32_t *z,
                                       uint32_t *v) {
  const uint32_t idx = index[q];
  *x = (int32_t)(idx % width);
  *y = (int32_t)(idx / width);
  *z = frame[q];
  *v = value[q];
}

// The reference's emit() (dials_spots.cc:240-353) over members sorted into
// (frame, index) order: the first pass from exact integers when they are
// exact (else the double sequence), then the variance pass sequentially in
// double, the same operations in the same order as the reference. The
// variance pass is skipped when only acceptance is wanted. Returns false if
// the peak-centroid filter rejects the spot.
__device__ bool emit_spot(const uint32_t *mem, uint32_t n, const int32_t *frame,
                          const uint32_t *index, const uint32_t *value, uint32_t width,
                          double max_separation, sf_spot *spot, bool variance = true,
                          const FirstPass *given = nullptr) {
  FirstPass f;
  if (given) {
    f = *given;
  } else {
    fp_init(f);
    for (uint32_t k = 0; k < n; k++) {
      int32_t x, y, z;
      uint32_t v;
      member(mem[k], frame, index, value, width, &x, &y, &z, &v);
      fp_add(f, k, v, x, y, z);
    }
    fp_finish(f);
  }
  double sum, sum_sq, weighted[3], peak[3];
  if (f.exact) {
    sum = (double)f.S;
    sum_sq = (double)f.Q2;
    for (int ax = 0; ax < 3; ax++)
      weighted[ax] = __dmul_rn((double)f.W[ax], 0.5);  // exact: W < 2^53
    peak[0] = peak[1] = peak[2] = 0.0;
    if (f.peak_k != 0xFFFFFFFFu) {
      int32_t px, py, pz;
      uint32_t pv;
      member(mem[f.peak_k], frame, index, value, width, &px, &py, &pz, &pv);
      peak[0] = __dadd_rn((double)px, 0.5);
      peak[1] = __dadd_rn((double)py, 0.5);
      peak[2] = __dadd_rn((double)pz, 0.5);
    }
  } else {
    sum = sum_sq = 0.0;
    weighted[0] = weighted[1] = weighted[2] = 0.0;
    peak[0] = peak[1] = peak[2] = 0.0;
    uint32_t peak_value = 0;
    for (uint32_t k = 0; k < n; k++) {
      int32_t x, y, z;
      uint32_t v;
      member(mem[k], frame, index, value, width, &x, &y, &z, &v);
      const double val = (double)v;
      const double pos[3] = {__dadd_rn((double)x, 0.5), __dadd_rn((double)y, 0.5),
                             __dadd_rn((double)z, 0.5)};
      sum = __dadd_rn(sum, val);
      sum_sq = __dadd_rn(sum_sq, __dmul_rn(val, val));
      for (int ax = 0; ax < 3; ax++)
        weighted[ax] = __dadd_rn(weighted[ax], __dmul_rn(val, pos[ax]));
      if (v > peak_value) {
        peak_value = v;
        peak[0] = pos[0], peak[1] = pos[1], peak[2] = pos[2];
      }
    }
  }
  sf_spot s;
  for (int a = 0; a < 6; a++)
    s.bbox[a] = f.bb[a];
  s.intensity = sum;
  s.intensity_variance = sum;
  s.n_signal = n;
  s.first = 0;
  s.variance[0] = s.variance[1] = s.variance[2] = 0.0;
  const double pixel_variance = 1.0 / 12.0;
  if (sum > 0.0) {
    for (int ax = 0; ax < 3; ax++)
      s.position[ax] = __ddiv_rn(weighted[ax], sum);
    if (variance) {
      double delta_sq[3] = {0.0, 0.0, 0.0};
      for (uint32_t k = 0; k < n; k++) {
        int32_t x, y, z;
        uint32_t v;
        member(mem[k], frame, index, value, width, &x, &y, &z, &v);
        const double val = (double)v;
        const double pos[3] = {__dadd_rn((double)x, 0.5), __dadd_rn((double)y, 0.5),
                               __dadd_rn((double)z, 0.5)};
        for (int ax = 0; ax < 3; ax++) {
          const double d = __dsub_rn(pos[ax], s.position[ax]);
          delta_sq[ax] = __dadd_rn(delta_sq[ax], __dmul_rn(__dmul_rn(val, d), d));
        }
      }
      const double ss = __dmul_rn(sum, sum);
      if (ss > sum_sq) {
        for (int ax = 0; ax < 3; ax++) {
          const double var = __ddiv_rn(__dmul_rn(delta_sq[ax], sum), __dsub_rn(ss, sum_sq));
          s.variance[ax] = __dadd_rn(__ddiv_rn(var, sum), pixel_variance);
        }
      } else {
        for (int ax = 0; ax < 3; ax++)
          s.variance[ax] = pixel_variance;
      }
    }
    if (s.bbox[5] == s.bbox[4] + 1)
      s.position[2] = __dadd_rn((double)s.bbox[4], 0.5);
  } else {
    s.position[0] = __ddiv_rn((double)(s.bbox[1] + s.bbox[0]), 2.0);
    s.position[1] = __ddiv_rn((double)(s.bbox[3] + s.bbox[2]), 2.0);
    s.position[2] = __ddiv_rn((double)(s.bbox[5] + s.bbox[4]), 2.0);
  }
  *spot = s;
  if (max_separation > 0.0) {
    const double dx = __dsub_rn(peak[0], s.position[0]);
    const double dy = __dsub_rn(peak[1], s.position[1]);
    const double dz = __dsub_rn(peak[2], s.position[2]);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (__dsqrt_rn(d2) > max_separation)
      return false;
  }
  return true;
}

// One warp per candidate of up to kWarpSortMax members (or one block per
// candidate of up to kBlockSortMax): sort the members into (frame, index)
// order, write them back, run emit() and record acceptance.
template <bool BLOCK>
__global__ void __launch_bounds__(kThreads)
k_sort_accept(LabelStatus *st, const BatchArgs *__restrict__ ap,
              const uint32_t *__restrict__ cand_n,
              const uint32_t *__restrict__ cand_off, uint32_t *members,
              const int32_t *__restrict__ frame, const uint32_t *__restrict__ index,
              const uint32_t *__restrict__ value, uint32_t *acc, uint32_t *acc_n) {
  const BatchArgs &a = *ap;
  if (st->error)
    return;
  extern __shared__ __align__(16) uint32_t s_sort[];
  const uint32_t ncand = st->n_cand;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  uint32_t separated = 0;
  if (!BLOCK) {
    uint32_t *s = s_sort + warp * kWarpSortMax;
    for (uint32_t c = blockIdx.x * nwarps + warp; c < ncand; c += gridDim.x * nwarps) {
      const uint32_t n = cand_n[c];
      if (n > (uint32_t)kWarpSortMax)
        continue;
      uint32_t *m = members + cand_off[c];
      for (uint32_t i = lane; i < n; i += 32)
        s[i] = m[i];
      __syncwarp();
      bitonic_sort(s, (int)n, lane, 32, true);
      for (uint32_t i = lane; i < n; i += 32)
        m[i] = s[i];
      // The first pass across the warp, exact in integers.
      FirstPass f;
      fp_init(f);
      for (uint32_t i = lane; i < n; i += 32) {
        int32_t x, y, z;
        uint32_t v;
        member(s[i], frame, index, value, a.width, &x, &y, &z, &v);
        fp_add(f, i, v, x, y, z);
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        FirstPass g;
        g.S = __shfl_xor_sync(0xffffffffu, f.S, o);
        g.Q2 = __shfl_xor_sync(0xffffffffu, f.Q2, o);
        for (int ax = 0; ax < 3; ax++)
          g.W[ax] = __shfl_xor_sync(0xffffffffu, f.W[ax], o);
        for (int b = 0; b < 6; b++)
          g.bb[b] = __shfl_xor_sync(0xffffffffu, f.bb[b], o);
        g.peak_v = __shfl_xor_sync(0xffffffffu, f.peak_v, o);
        g.peak_k = __shfl_xor_sync(0xffffffffu, f.peak_k, o);
        g.exact = __shfl_xor_sync(0xffffffffu, f.exact ? 1 : 0, o) != 0;
        fp_merge(f, g);
      }
      __syncwarp();
      if (lane == 0) {
        fp_finish(f);
        sf_spot spot;
        const bool ok = emit_spot(s, n, frame, index, value, a.width, a.max_separation, &spot,
                                  false, f.exact ? &f : nullptr);
        acc[c] = ok ? 1u : 0u;
        acc_n[c] = ok ? n : 0u;
        separated += ok ? 0u : 1u;
      }
      __syncwarp();
    }
  } else {
    __shared__ sf_spot s_spot;
    __shared__ uint32_t s_ok;
    for (uint32_t c = blockIdx.x; c < ncand; c += gridDim.x) {
      const uint32_t n = cand_n[c];
      if (n <= (uint32_t)kWarpSortMax)
        continue;
      if (n > (uint32_t)kBlockSortMax) {
        if (threadIdx.x == 0) {
          atomicOr(&st->error, kErrSpotSize);
          acc[c] = 0;
          acc_n[c] = 0;
        }
        continue;
      }
      uint32_t *m = members + cand_off[c];
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        s_sort[i] = m[i];
      __syncthreads();
      bitonic_sort(s_sort, (int)n, threadIdx.x, blockDim.x, false);
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        m[i] = s_sort[i];
      if (threadIdx.x == 0) {
        s_ok = emit_spot(s_sort, n, frame, index, value, a.width, a.max_separation, &s_spot,
                         false)
                   ? 1u : 0u;
        acc[c] = s_ok;
        acc_n[c] = s_ok ? n : 0u;
        separated += s_ok ? 0u : 1u;
      }
      __syncthreads();
    }
  }
  if (separated)
    atomicAdd(&st->counts[kCntSeparated], (unsigned long long)separated);
}

// Accepted spots and their pixels into the batch outputs (dials_spots.cc:
// 355-359): spot k's pixels at acc_off[k] in member order. Four lanes to a
// candidate: the first pass split four ways (exact integers), then each of
// three lanes runs one axis of the variance pass -- a sequence of rounded
// double additions in member order, as the reference -- and lane 0 writes
// the spot. Where the integers could be inexact lane 0 runs the whole
// reference sequence alone.
__global__ void __launch_bounds__(kThreads)
k_write(LabelStatus *st, const BatchArgs *__restrict__ ap,
        const uint32_t *__restrict__ cand_n,
        const uint32_t *__restrict__ cand_off, const uint32_t *__restrict__ members,
        const int32_t *__restrict__ frame, const uint32_t *__restrict__ index,
        const uint32_t *__restrict__ value, const uint32_t *__restrict__ acc,
        const uint32_t *__restrict__ acc_idx, const uint32_t *__restrict__ acc_off,
        sf_spot *spots, size_t spots_cap, sf_pixel *pixels, size_t pixels_cap) {
  const BatchArgs &a = *ap;
  if (st->error)
    return;
  const uint32_t ncand = st->n_cand;
  const int lane = threadIdx.x & 31, sub = lane & 3;
  const uint32_t per_pass = (gridDim.x * blockDim.x) >> 2;
  for (uint32_t base = (blockIdx.x * blockDim.x) >> 2; base < ncand; base += per_pass) {
    const uint32_t c = base + (threadIdx.x >> 2);
    bool live = c < ncand && acc[c];
    uint32_t n = 0, si = 0, po = 0;
    const uint32_t *m = nullptr;
    if (live) {
      n = cand_n[c];
      si = acc_idx[c];
      po = acc_off[c];
      m = members + cand_off[c];
      if (si >= spots_cap || (size_t)po + n > pixels_cap) {
        if (sub == 0)
          atomicOr(&st->error, kErrOutFull);
        live = false;
      }
    }
    FirstPass f;
    fp_init(f);
    if (live)
      for (uint32_t k = sub; k < n; k += 4) {
        const uint32_t q = m[k];
        int32_t x, y, z;
        uint32_t v;
        member(q, frame, index, value, a.width, &x, &y, &z, &v);
        fp_add(f, k, v, x, y, z);
        sf_pixel px;
        px.frame = z;
        px.index = index[q];
        px.value = v;
        pixels[po + k] = px;
      }
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
      FirstPass g;
      g.S = __shfl_xor_sync(0xffffffffu, f.S, o);
      g.Q2 = __shfl_xor_sync(0xffffffffu, f.Q2, o);
      for (int ax = 0; ax < 3; ax++)
        g.W[ax] = __shfl_xor_sync(0xffffffffu, f.W[ax], o);
      for (int bb = 0; bb < 6; bb++)
        g.bb[bb] = __shfl_xor_sync(0xffffffffu, f.bb[bb], o);
      g.peak_v = __shfl_xor_sync(0xffffffffu, f.peak_v, o);
      g.peak_k = __shfl_xor_sync(0xffffffffu, f.peak_k, o);
      g.exact = __shfl_xor_sync(0xffffffffu, f.exact ? 1 : 0, o) != 0;
      fp_merge(f, g);
    }
    fp_finish(f);
    double var_ax = 0.0;
    sf_spot spot;
    if (live && f.exact) {
      // This lane's axis of the variance pass (lanes 0, 1, 2).
      const double sum = (double)f.S, sum_sq = (double)f.Q2;
      double pos_c[3];
      for (int ax = 0; ax < 3; ax++)
        pos_c[ax] = __ddiv_rn(__dmul_rn((double)f.W[ax], 0.5), sum);
      if (sub < 3 && sum > 0.0) {
        double delta_sq = 0.0;
        const double centre = pos_c[sub];
        for (uint32_t k = 0; k < n; k++) {
          const uint32_t q = m[k];
          int32_t x, y, z;
          uint32_t v;
          member(q, frame, index, value, a.width, &x, &y, &z, &v);
          const int32_t coord = sub == 0 ? x : sub == 1 ? y : z;
          const double d = __dsub_rn(__dadd_rn((double)coord, 0.5), centre);
          delta_sq = __dadd_rn(delta_sq, __dmul_rn(__dmul_rn((double)v, d), d));
        }
        const double ss = __dmul_rn(sum, sum);
        var_ax = ss > sum_sq
                     ? __dadd_rn(__ddiv_rn(__ddiv_rn(__dmul_rn(delta_sq, sum),
                                                     __dsub_rn(ss, sum_sq)),
                                           sum),
                                 1.0 / 12.0)
                     : 1.0 / 12.0;
      }
      for (int b6 = 0; b6 < 6; b6++)
        spot.bbox[b6] = f.bb[b6];
      spot.intensity = sum;
      spot.intensity_variance = sum;
      spot.n_signal = n;
      if (sum > 0.0) {
        spot.position[0] = pos_c[0];
        spot.position[1] = pos_c[1];
        spot.position[2] = spot.bbox[5] == spot.bbox[4] + 1
                               ? __dadd_rn((double)spot.bbox[4], 0.5) : pos_c[2];
      } else {
        spot.position[0] = __ddiv_rn((double)(spot.bbox[1] + spot.bbox[0]), 2.0);
        spot.position[1] = __ddiv_rn((double)(spot.bbox[3] + spot.bbox[2]), 2.0);
        spot.position[2] = __ddiv_rn((double)(spot.bbox[5] + spot.bbox[4]), 2.0);
      }
    }
    // Lane 0 of each group gathers the three axes' variances.
    const double v1 = __shfl_down_sync(0xffffffffu, var_ax, 1);
    const double v2 = __shfl_down_sync(0xffffffffu, var_ax, 2);
    if (live && sub == 0) {
      if (f.exact) {
        const bool spread = (double)f.S > 0.0;
        spot.variance[0] = spread ? var_ax : 0.0;
        spot.variance[1] = spread ? v1 : 0.0;
        spot.variance[2] = spread ? v2 : 0.0;
      } else {
        emit_spot(m, n, frame, index, value, a.width, a.max_separation, &spot);
      }
      spot.first = a.pixel_base + po;
      spots[si] = spot;
    }
  }
}

__global__ void k_compact(LabelStatus *st, const uint32_t *__restrict__ open,
                          const uint32_t *__restrict__ newpos,
                          const uint32_t *__restrict__ root, const int32_t *__restrict__ frame,
                          const uint32_t *__restrict__ index, const uint32_t *__restrict__ value,
                          int32_t *frame2, uint32_t *index2, uint32_t *value2,
                          uint32_t *parent2) {
  if (st->error)
    return;
  const uint32_t n = st->n_total;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += gridDim.x * blockDim.x) {
    if (open[p]) {
      const uint32_t q = newpos[p];
      frame2[q] = frame[p];
      index2[q] = index[p];
      value2[q] = value[p];
      parent2[q] = newpos[root[p]];
    }
  }
}

__global__ void k_end_batch(LabelStatus *st, const BatchArgs *__restrict__ ap) {
  const BatchArgs &a = *ap;
  if (threadIdx.x != 0 || st->error)
    return;
  st->counts[kCntAccepted] += st->n_accept;
  st->n_live = st->n_open;
  if (st->n_open == 0) {
    st->prev_start = 0;
  } else {
    // Every pixel of the last frame belongs to a component still open, and
    // they are the tail of the pool (dials_spots.cc:378-380).
    const uint32_t last = st->frame_off[a.nb] - st->frame_off[a.nb - 1];
    st->prev_start = st->n_open - last;
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------

template <typename T> static cudaError_t dalloc(T **p, size_t n) {
  return cudaMalloc(reinterpret_cast<void **>(p), (n ? n : 1) * sizeof(T));
}

// The run's spots and kept pixels, append-only in device memory, in chunks
// that never move (1 MiB first, doubling to 256 MiB): a batch's outputs are
// appended by device-to-device copies on its stream, and nothing is copied to
// the host until a caller asks. Growing a host array instead meant pinning
// and copying ever larger buffers on the labelling thread.
template <typename T> struct DeviceStore {
  struct Chunk {
    T *p;
    size_t cap;
  };
  std::vector<Chunk> chunks;
  size_t n = 0, cap = 0;
  DeviceStore() = default;
  DeviceStore(const DeviceStore &) = delete;
  DeviceStore &operator=(const DeviceStore &) = delete;
  ~DeviceStore() {
    for (const Chunk &c : chunks)
      cudaFree(c.p);
  }
  size_t size() const { return n; }
  // Room for m more elements.
  cudaError_t reserve_more(size_t m) {
    constexpr size_t kFirst = (size_t(1) << 20) / sizeof(T) + 1;
    constexpr size_t kMax = (size_t(256) << 20) / sizeof(T);
    while (cap < n + m) {
      size_t c = chunks.empty() ? kFirst : std::min(chunks.back().cap * 2, kMax);
      c = std::max(c, std::min(n + m - cap, kMax));
      T *q = nullptr;
      const cudaError_t e = cudaMalloc(&q, c * sizeof(T));
      if (e != cudaSuccess)
        return e;
      chunks.push_back({q, c});
      cap += c;
    }
    return cudaSuccess;
  }
  // Visit [from, from + m) as pieces (chunk pointer, element offset in the run,
  // length).
  template <typename F> cudaError_t pieces(size_t from, size_t m, F f) const {
    size_t base = 0;
    for (const Chunk &c : chunks) {
      if (m == 0)
        break;
      if (from < base + c.cap) {
        const size_t off = from - base, take = std::min(c.cap - off, m);
        const cudaError_t e = f(c.p + off, from, take);
        if (e != cudaSuccess)
          return e;
        from += take;
        m -= take;
      }
      base += c.cap;
    }
    return cudaSuccess;
  }
  cudaError_t append(const T *src, size_t m, cudaStream_t s) {
    cudaError_t e = reserve_more(m);
    if (e != cudaSuccess || m == 0)
      return e;
    const size_t at = n;
    e = pieces(at, m, [&](T *dst, size_t pos, size_t len) {
      return cudaMemcpyAsync(dst, src + (pos - at), len * sizeof(T), cudaMemcpyDeviceToDevice, s);
    });
    if (e == cudaSuccess)
      n += m;
    return e;
  }
  // Everything stored, into host memory, on stream s (synchronised).
  cudaError_t read(T *out, cudaStream_t s) const {
    cudaError_t e = pieces(0, n, [&](T *src, size_t pos, size_t len) {
      return cudaMemcpyAsync(out + pos, src, len * sizeof(T), cudaMemcpyDeviceToHost, s);
    });
    return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
  }
};

struct Labeller {
  size_t height = 0, width = 0, capacity = 0, spots_cap = 0;
  sf_label_options opt;
  cudaStream_t own_stream = nullptr;
  bool started = false;
  int64_t last_frame = 0;
  bool finished = false;
  // Live pool, ping-pong.
  int32_t *frame[2] = {nullptr, nullptr};
  uint32_t *index[2] = {nullptr, nullptr}, *value[2] = {nullptr, nullptr};
  uint32_t *parent[2] = {nullptr, nullptr};
  int cur = 0;
  // Scratch sized by capacity.
  uint32_t *root = nullptr, *csize = nullptr, *candid = nullptr, *flag = nullptr,
           *open = nullptr, *posa = nullptr, *posb = nullptr, *clist = nullptr,
           *cbucket = nullptr, *order = nullptr, *cflag = nullptr, *cpos = nullptr,
           *cand_root = nullptr, *cand_n = nullptr, *cand_off = nullptr, *cursor = nullptr,
           *members = nullptr, *acc = nullptr, *acc_n = nullptr, *acc_idx = nullptr,
           *acc_off = nullptr, *hist = nullptr, *block_sums = nullptr;
  int32_t *zlast = nullptr;
  LabelStatus *st = nullptr;
  LabelStatus *host_st = nullptr;
  BatchArgs *d_args = nullptr, *h_args = nullptr;
  // Captured launch sequences by (live pool, frames in the batch).
  cudaGraphExec_t graphs[2][kLabelMaxBatch + 1] = {};
  bool seen[2][kLabelMaxBatch + 1] = {};
  bool use_graphs = true;
  // Batch outputs, copied to the host vectors after every batch.
  sf_spot *d_spots = nullptr;
  sf_pixel *d_pixels = nullptr;
  // Host-list upload staging.
  sf_signal_pixel *d_list = nullptr;
  size_t d_list_cap = 0;
  uint32_t *d_counts = nullptr;
  DeviceStore<sf_spot> spots;
  DeviceStore<sf_pixel> pixels;
  // Recorded after each call's appends: the next call (on whatever stream)
  // and the readers wait for it before touching the batch outputs or the
  // stores.
  cudaEvent_t appended = nullptr;
  sf_counts counts{};
  uint32_t live = 0;
  std::string error;

  ~Labeller() {
    if (own_stream) {
      cudaStreamSynchronize(own_stream);
      cudaStreamDestroy(own_stream);
    }
    for (int i = 0; i < 2; i++) {
      cudaFree(frame[i]);
      cudaFree(index[i]);
      cudaFree(value[i]);
      cudaFree(parent[i]);
    }
    uint32_t *bufs[] = {root, csize, candid, flag, open, posa, posb, clist, cbucket,
                        order, cflag, cpos, cand_root, cand_n, cand_off, cursor,
                        members, acc, acc_n, acc_idx, acc_off, hist, block_sums, d_counts};
    for (uint32_t *b : bufs)
      cudaFree(b);
    for (auto &row : graphs)
      for (cudaGraphExec_t g : row)
        if (g)
          cudaGraphExecDestroy(g);
    cudaFree(zlast);
    cudaFree(st);
    cudaFree(d_args);
    if (h_args)
      cudaFreeHost(h_args);
    cudaFree(d_spots);
    cudaFree(d_pixels);
    cudaFree(d_list);
    if (host_st)
      cudaFreeHost(host_st);
    if (appended)
      cudaEventDestroy(appended);
  }

  int init() {
    cudaError_t e;
    const size_t n = capacity;
#define SF_ALLOC(ptr, cnt)                                                               \
  if ((e = dalloc(&(ptr), (cnt))) != cudaSuccess)                                        \
    return fail(e, "cudaMalloc for the labeller");
    for (int i = 0; i < 2; i++) {
      SF_ALLOC(frame[i], n);
      SF_ALLOC(index[i], n);
      SF_ALLOC(value[i], n);
      SF_ALLOC(parent[i], n);
    }
    SF_ALLOC(root, n);
    SF_ALLOC(csize, n);
    SF_ALLOC(candid, n);
    SF_ALLOC(flag, n);
    SF_ALLOC(open, n);
    SF_ALLOC(posa, n);
    SF_ALLOC(posb, n);
    SF_ALLOC(clist, n);
    SF_ALLOC(cbucket, n);
    SF_ALLOC(order, n);
    SF_ALLOC(cflag, n);
    SF_ALLOC(cpos, n);
    SF_ALLOC(cand_root, n);
    SF_ALLOC(cand_n, n);
    SF_ALLOC(cand_off, n);
    SF_ALLOC(cursor, n);
    SF_ALLOC(members, n);
    SF_ALLOC(acc, n);
    SF_ALLOC(acc_n, n);
    SF_ALLOC(acc_idx, n);
    SF_ALLOC(acc_off, n);
    SF_ALLOC(hist, (size_t)kGrid * kBuckets);
    SF_ALLOC(block_sums, kScanBlocks);
    SF_ALLOC(zlast, n);
    // At most one accepted spot per min_spot_size pixels closed in a batch.
    spots_cap = n / (opt.min_spot_size ? opt.min_spot_size : 1) + 1;
    SF_ALLOC(d_spots, spots_cap);
    SF_ALLOC(d_pixels, n);
    SF_ALLOC(d_counts, kLabelMaxBatch);
#undef SF_ALLOC
    if ((e = cudaMalloc(&st, sizeof(LabelStatus))) != cudaSuccess)
      return fail(e, "cudaMalloc for the labeller status");
    if ((e = cudaMallocHost(&host_st, sizeof(LabelStatus))) != cudaSuccess)
      return fail(e, "cudaMallocHost for the labeller status");
    if ((e = cudaEventCreateWithFlags(&appended, cudaEventDisableTiming)) != cudaSuccess)
      return fail(e, "cudaEventCreate");
    if ((e = cudaMalloc(&d_args, sizeof(BatchArgs))) != cudaSuccess)
      return fail(e, "cudaMalloc for the labeller's arguments");
    if ((e = cudaMallocHost(&h_args, sizeof(BatchArgs))) != cudaSuccess)
      return fail(e, "cudaMallocHost for the labeller's arguments");
    if ((e = cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking)) != cudaSuccess)
      return fail(e, "cudaStreamCreate");
    if ((e = cudaMemsetAsync(st, 0, sizeof(LabelStatus), own_stream)) != cudaSuccess)
      return fail(e, "clearing the labeller status");
    if ((e = cudaStreamSynchronize(own_stream)) != cudaSuccess)
      return fail(e, "cudaStreamSynchronize");
    return SF_OK;
  }

  // The launch sequence of one batch of nb frames on stream s, reading the
  // call's arguments from d_args; pool c is the live pool, 1 - c the next.
  cudaError_t enqueue(int nb, int c, cudaStream_t s) {
    const int o = 1 - c;
    const BatchArgs *ap = d_args;
    const dim3 g2(kGrid / 4 > 0 ? kGrid / 4 : 1, nb);
    cudaError_t e;
    k_offsets<<<1, 32, 0, s>>>(st, ap, (uint32_t)capacity);
    k_append<<<g2, kThreads, 0, s>>>(st, ap, frame[c], index[c], value[c], parent[c]);
    k_link<<<g2, kThreads, 0, s>>>(st, ap, index[c], parent[c]);
    k_flatten<<<kGrid, kThreads, 0, s>>>(st, parent[c], root, zlast, csize, candid);
    k_comp_stats<<<kGrid, kThreads, 0, s>>>(st, root, frame[c], zlast, csize);
    k_closing_flags<<<kGrid, kThreads, 0, s>>>(st, ap, root, zlast, flag, open);
    const uint32_t *err = &st->error;
    if ((e = exclusive_scan(flag, posa, &st->n_total, &st->n_closing, block_sums, err, s)) !=
        cudaSuccess)
      return e;
    k_closing_list<<<kGrid, kThreads, 0, s>>>(st, ap, flag, posa, zlast, clist, cbucket);
    k_bucket_hist<<<kGrid, kThreads, 0, s>>>(st, cbucket, hist);
    k_bucket_offsets<<<1, 128, 0, s>>>(st, hist);
    k_bucket_scatter<<<kGrid, kThreads, 0, s>>>(st, clist, cbucket, hist, order);
    k_size_filter<<<kGrid, kThreads, 0, s>>>(st, ap, order, csize, cflag);
    if ((e = exclusive_scan(cflag, cpos, &st->n_closing, &st->n_cand, block_sums, err, s)) !=
        cudaSuccess)
      return e;
    k_cand_list<<<kGrid, kThreads, 0, s>>>(st, order, csize, cflag, cpos, cand_root, cand_n,
                                           candid, cursor);
    if ((e = exclusive_scan(cand_n, cand_off, &st->n_cand, &st->n_cand_pixels, block_sums,
                            err, s)) != cudaSuccess)
      return e;
    k_gather<<<kGrid, kThreads, 0, s>>>(st, root, candid, cand_off, cursor, members);
    k_sort_accept<false><<<kGrid, kThreads, (kThreads / 32) * kWarpSortMax * 4, s>>>(
        st, ap, cand_n, cand_off, members, frame[c], index[c], value[c], acc, acc_n);
    k_sort_accept<true><<<kGrid / 2, kThreads, kBlockSortMax * 4, s>>>(
        st, ap, cand_n, cand_off, members, frame[c], index[c], value[c], acc, acc_n);
    if ((e = exclusive_scan(acc, acc_idx, &st->n_cand, &st->n_accept, block_sums, err, s)) !=
        cudaSuccess)
      return e;
    if ((e = exclusive_scan(acc_n, acc_off, &st->n_cand, &st->n_accept_pixels, block_sums,
                            err, s)) != cudaSuccess)
      return e;
    k_write<<<kGrid, kThreads, 0, s>>>(st, ap, cand_n, cand_off, members, frame[c], index[c],
                                       value[c], acc, acc_idx, acc_off, d_spots, spots_cap,
                                       d_pixels, capacity);
    if ((e = exclusive_scan(open, posb, &st->n_total, &st->n_open, block_sums, err, s)) !=
        cudaSuccess)
      return e;
    k_compact<<<kGrid, kThreads, 0, s>>>(st, open, posb, root, frame[c], index[c], value[c],
                                         frame[o], index[o], value[o], parent[o]);
    k_end_batch<<<1, 32, 0, s>>>(st, ap);
    return cudaGetLastError();
  }

  // The sequence for (nb, c) as a CUDA graph, captured on the labeller's own
  // stream the second time that shape is met (the first runs directly, so
  // every kernel is loaded before a capture), then replayed on any stream.
  // Null if capture is not possible (the caller's stream is itself being
  // captured, or the capture failed): the sequence then runs directly.
  cudaGraphExec_t graph_for(int nb, int c, cudaStream_t s) {
    cudaGraphExec_t &g = graphs[c][nb];
    if (g || !use_graphs)
      return g;
    if (!seen[c][nb]) {
      seen[c][nb] = true;
      return nullptr;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (s != cudaStreamLegacy && cudaStreamIsCapturing(s, &cs) == cudaSuccess &&
        cs != cudaStreamCaptureStatusNone)
      return nullptr;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(own_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    const cudaError_t e = enqueue(nb, c, own_stream);
    const cudaError_t e2 = cudaStreamEndCapture(own_stream, &graph);
    if (e == cudaSuccess && e2 == cudaSuccess && graph &&
        cudaGraphInstantiate(&g, graph, 0) != cudaSuccess)
      g = nullptr;
    if (graph)
      cudaGraphDestroy(graph);
    if (!g) {
      use_graphs = false;  // do not try again
      cudaGetLastError();
    }
    return g;
  }

  // One batch: frames[j]'s list at lists + j * stride, count counts[j].
  int run_batch(const int64_t *frames, int nb, const sf_signal_pixel *lists,
                size_t stride, const uint32_t *counts_dev, bool finishing,
                cudaStream_t s) {
    BatchArgs &a = *h_args;
    std::memset(&a, 0, sizeof(a));
    a.lists = lists;
    a.counts = counts_dev;
    a.stride = stride;
    a.pixel_base = pixels.size();
    a.nb = nb;
    a.finishing = finishing ? 1 : 0;
    a.two_d = opt.two_d ? 1 : 0;
    a.width = (uint32_t)width;
    a.npix = (uint32_t)(height * width);
    a.min_size = (uint32_t)std::min<size_t>(opt.min_spot_size, 0xffffffffu);
    a.max_size = (uint32_t)std::min<size_t>(opt.max_spot_size, 0xffffffffu);
    a.max_separation = opt.max_separation;
    int64_t prev = last_frame;
    bool have_prev = started;
    for (int j = 0; j < nb; j++) {
      a.frames[j] = (int32_t)frames[j];
      a.link_prev[j] = (!opt.two_d && have_prev && frames[j] == prev + 1) ? 1 : 0;
      prev = frames[j];
      have_prev = true;
    }
    if (nb == 0) { // finish(): one flush of everything, nothing appended
      a.nb = 1;
      a.frames[0] = (int32_t)(last_frame + 1);
      a.link_prev[0] = 0;
    }
    // h_args is reused by the next call only after collect() has waited for
    // this one, so the copy has read it by then.
    cudaError_t e;
    if ((e = cudaStreamWaitEvent(s, appended, 0)) != cudaSuccess)
      return fail(e, "cudaStreamWaitEvent");
    if ((e = cudaMemcpyAsync(d_args, h_args, sizeof(BatchArgs), cudaMemcpyHostToDevice, s)) !=
        cudaSuccess)
      return fail(e, "copying the labeller's arguments");
    if (cudaGraphExec_t g = graph_for(a.nb, cur, s))
      e = cudaGraphLaunch(g, s);
    else
      e = enqueue(a.nb, cur, s);
    if (e != cudaSuccess)
      return fail(e, "launching the labeller");
    return collect(s, nb > 0 ? frames[nb - 1] : last_frame, nb > 0);
  }

  // Read the batch's status and outputs back and append them to the run.
  int collect(cudaStream_t s, int64_t newest, bool added) {
    cudaError_t e;
    if ((e = cudaMemcpyAsync(host_st, st, sizeof(LabelStatus), cudaMemcpyDeviceToHost, s)) !=
        cudaSuccess)
      return fail(e, "reading the labeller status");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess)
      return fail(e, "cudaStreamSynchronize");
    if (host_st->error) {
      const uint32_t err = host_st->error;
      t_last_error = (err & kErrLiveFull)
                         ? "more signal pixels held open at once than the labeller's "
                           "capacity"
                     : (err & kErrSpotSize)
                         ? "a spot within the size limits is larger than 8192 pixels"
                     : (err & kErrOutFull) ? "labeller outputs overflowed"
                     : (err & kErrListOverflow)
                         ? "a signal list's count exceeds its capacity (the threshold "
                           "overflowed)"
                         : "a union did not settle";
      return SF_EOVERFLOW;
    }
    const uint32_t na = host_st->n_accept, npx = host_st->n_accept_pixels;
    if ((e = spots.append(d_spots, na, s)) != cudaSuccess ||
        (e = pixels.append(d_pixels, npx, s)) != cudaSuccess)
      return fail(e, "storing the labeller's results");
    if ((e = cudaEventRecord(appended, s)) != cudaSuccess)
      return fail(e, "cudaEventRecord");
    const unsigned long long *c = host_st->counts;
    counts.signal_pixels = c[kCntSignal];
    counts.groups = c[kCntGroups];
    counts.too_small = c[kCntSmall];
    counts.too_large = c[kCntLarge];
    counts.separated = c[kCntSeparated];
    counts.accepted = c[kCntAccepted];
    live = host_st->n_live;
    cur = 1 - cur;
    if (added) {
      started = true;
      last_frame = newest;
    }
    return SF_OK;
  }
};

} // namespace sf

using namespace sf;

struct sf_labeller {
  Labeller impl;
};

// The stored results to the host, after the last call's appends.
template <typename T>
static int read_store(const Labeller &L, const DeviceStore<T> &v, T *out, size_t capacity,
                      const char *what) {
  if (capacity < v.size())
    return SF_EOVERFLOW;
  cudaError_t e;
  if ((e = cudaStreamWaitEvent(L.own_stream, L.appended, 0)) != cudaSuccess ||
      (e = v.read(out, L.own_stream)) != cudaSuccess)
    return fail(e, what);
  return SF_OK;
}

namespace sf {

size_t label_width(const sf_labeller *l) { return l ? l->impl.width : 0; }

int label_gather_pixels(const sf_labeller *l, sf_pixel *d_out, cudaStream_t *stream) {
  const Labeller &L = l->impl;
  *stream = L.own_stream;
  cudaError_t e = cudaStreamWaitEvent(L.own_stream, L.appended, 0);
  if (e == cudaSuccess)
    e = L.pixels.pieces(0, L.pixels.size(), [&](sf_pixel *src, size_t pos, size_t len) {
      return cudaMemcpyAsync(d_out + pos, src, len * sizeof(sf_pixel), cudaMemcpyDeviceToDevice,
                             L.own_stream);
    });
  return e == cudaSuccess ? SF_OK : fail(e, "gathering the spot pixels");
}

} // namespace sf

extern "C" {

void sf_default_label_options(sf_label_options *o) {
  if (!o)
    return;
  o->min_spot_size = 3;
  o->max_spot_size = 1000;
  o->max_separation = 2.0;
  o->two_d = 0;
}

sf_labeller *sf_label_open(size_t height, size_t width, const sf_label_options *options,
                           size_t live_capacity) {
  sf_label_options o;
  if (options)
    o = *options;
  else
    sf_default_label_options(&o);
  // dials_spots.cc:21-30
  if (height == 0 || width == 0 || height > 0x7fffffffu / width) {
    t_last_error = "dials_spots: a frame with no pixels in it";
    return nullptr;
  }
  if (o.max_spot_size < o.min_spot_size) {
    t_last_error = "max_spot_size is below min_spot_size, so nothing can be accepted";
    return nullptr;
  }
  if (o.min_spot_size == 0) {
    t_last_error = "min_spot_size must be at least 1";
    return nullptr;
  }
  sf_labeller *l = new (std::nothrow) sf_labeller;
  if (!l)
    return nullptr;
  l->impl.height = height;
  l->impl.width = width;
  l->impl.opt = o;
  l->impl.capacity = live_capacity ? live_capacity : (size_t)(1u << 22);
  if (l->impl.capacity > 0x7fffffffu)
    l->impl.capacity = 0x7fffffffu;
  if (l->impl.init() != SF_OK) {
    delete l;
    return nullptr;
  }
  return l;
}

void sf_label_close(sf_labeller *l) { delete l; }

int sf_label_add(sf_labeller *l, int64_t frame, const sf_signal_pixel *signal, size_t n) {
  if (!l || (!signal && n))
    return SF_EBADARG;
  Labeller &L = l->impl;
  // dials_spots.cc:58-63, :79-95: order and range checks, on the host.
  if (L.finished || (L.started && frame <= L.last_frame)) {
    t_last_error = "frames must be added in ascending order";
    return SF_EBADARG;
  }
  const uint64_t npix = (uint64_t)L.height * L.width;
  for (size_t i = 0; i < n; i++) {
    if (signal[i].index >= npix || (i && signal[i].index <= signal[i - 1].index)) {
      t_last_error = "signal pixels off the frame or not ascending by index";
      return SF_EBADARG;
    }
  }
  cudaError_t e;
  if (n > L.d_list_cap) {
    cudaFree(L.d_list);
    L.d_list = nullptr;
    L.d_list_cap = 0;
    if ((e = cudaMalloc(&L.d_list, n * sizeof(sf_signal_pixel))) != cudaSuccess)
      return fail(e, "cudaMalloc for the signal list");
    L.d_list_cap = n;
  }
  const uint32_t cnt = (uint32_t)n;
  if (n && (e = cudaMemcpyAsync(L.d_list, signal, n * sizeof(sf_signal_pixel),
                                cudaMemcpyHostToDevice, L.own_stream)) != cudaSuccess)
    return fail(e, "copying the signal list");
  if ((e = cudaMemcpyAsync(L.d_counts, &cnt, sizeof(uint32_t), cudaMemcpyHostToDevice,
                           L.own_stream)) != cudaSuccess)
    return fail(e, "copying the count");
  return L.run_batch(&frame, 1, L.d_list, n, L.d_counts, false, L.own_stream);
}

int sf_label_add_device(sf_labeller *l, const int64_t *frames, size_t n_frames,
                        const sf_signal_pixel *d_lists, size_t list_stride,
                        const uint32_t *d_counts, void *stream) {
  if (!l || !frames || !d_lists || !d_counts || n_frames == 0 ||
      n_frames > (size_t)kLabelMaxBatch)
    return SF_EBADARG;
  Labeller &L = l->impl;
  int64_t prev = L.last_frame;
  bool have = L.started;
  if (L.finished)
    return SF_EBADARG;
  for (size_t j = 0; j < n_frames; j++) {
    if (have && frames[j] <= prev) {
      t_last_error = "frames must be added in ascending order";
      return SF_EBADARG;
    }
    prev = frames[j];
    have = true;
  }
  // The stream the lists were produced on; NULL is the legacy default stream,
  // as for the threshold's device entry points.
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : cudaStreamLegacy;
  return L.run_batch(frames, (int)n_frames, d_lists, list_stride, d_counts, false, s);
}

int sf_label_finish(sf_labeller *l) {
  if (!l)
    return SF_EBADARG;
  Labeller &L = l->impl;
  if (L.finished || !L.started) {
    L.finished = true;
    return SF_OK;
  }
  cudaError_t e;
  const uint32_t zero = 0;
  if ((e = cudaMemcpyAsync(L.d_counts, &zero, sizeof(uint32_t), cudaMemcpyHostToDevice,
                           L.own_stream)) != cudaSuccess)
    return fail(e, "copying the count");
  const int rc = L.run_batch(nullptr, 0, L.d_list ? L.d_list : nullptr, 0, L.d_counts, true,
                             L.own_stream);
  L.finished = true;
  return rc;
}

size_t sf_label_n_spots(const sf_labeller *l) { return l ? l->impl.spots.size() : 0; }
size_t sf_label_n_pixels(const sf_labeller *l) { return l ? l->impl.pixels.size() : 0; }
size_t sf_label_live(const sf_labeller *l) { return l ? l->impl.live : 0; }

int sf_label_spots(const sf_labeller *l, sf_spot *out, size_t capacity) {
  if (!l || (!out && capacity))
    return SF_EBADARG;
  return read_store(l->impl, l->impl.spots, out, capacity, "reading spots back");
}

int sf_label_pixels(const sf_labeller *l, sf_pixel *out, size_t capacity) {
  if (!l || (!out && capacity))
    return SF_EBADARG;
  return read_store(l->impl, l->impl.pixels, out, capacity, "reading spot pixels back");
}

void sf_label_counts(const sf_labeller *l, sf_counts *out) {
  if (l && out)
    *out = l->impl.counts;
}

} // extern "C"
