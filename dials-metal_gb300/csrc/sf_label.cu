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

#include <algorithm>
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
constexpr int kGrid = 2 * 152;          // the bucket partition's chunks
constexpr int kPassGrid = 8 * 152;      // grid-stride passes over pixels / candidates
constexpr int kSortGrid = 6 * 152;      // warp sorts: 6 blocks an SM (registers)
constexpr int kWarpSortMax = 512;       // members ordered by one warp
constexpr int kWarpSegMax = 128;        // runs a warp orders without sorting the members
constexpr int kSegPerLane = kWarpSegMax / 32;
constexpr uint32_t kRunHead = 0x80000000u;  // a member slot's flag: the first of its run
constexpr uint32_t kPosMask = 0x7FFFFFFFu;  // a member slot's position (below 2^31)
constexpr int kBlockSortMax = 8192;     // members sorted by one block
constexpr int kUnionRetries = 1 << 20;  // cap on a union's CAS retries
// Frames up to this many rows get per-row start tables, so that a pixel's
// neighbours above and on the previous frame are searched for within one row
// of the ascending list instead of the whole frame.
constexpr uint32_t kRowTableMaxRows = 1u << 16;

enum : uint32_t {
  kErrLiveFull = 1u,   // more open pixels than the live pool holds
  kErrUnion = 2u,      // a union did not settle within kUnionRetries
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
  uint32_t n_big;       // candidates beyond a warp's sort, listed for the block sorts
  uint32_t n_edges;     // edges k_link listed for k_unite
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
  uint32_t wdiv_m, wdiv_s1, wdiv_s2;  // division by width (multiply-high)
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

// lower_bound with the same number of steps in every lane of the warp (the
// longest range's), so that the lanes stay together; all lanes call it.
__device__ __forceinline__ uint32_t lower_bound_warp(const uint32_t *__restrict__ v,
                                                     uint32_t lo, uint32_t hi, uint32_t key) {
  uint32_t len = hi - lo;
  const uint32_t longest = __reduce_max_sync(0xffffffffu, len);
  for (int steps = 32 - __clz(longest); steps > 0; steps--) {
    const uint32_t half = len >> 1;
    const bool right = len > 0 && v[lo + half] < key;
    lo = right ? lo + half + 1 : lo;
    len = right ? len - half - 1 : half;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// Kernels of one batch, in launch order.
// ---------------------------------------------------------------------------

// Each frame's offset in the batch, the exclusive prefix of the counts: one
// warp, frames 2l and 2l + 1 on lane l.
static_assert(kLabelMaxBatch <= 64, "two frames a lane");
__global__ void k_offsets(LabelStatus *st, const BatchArgs *__restrict__ ap,
                          uint32_t capacity) {
  if (st->error)
    return;
  const BatchArgs &a = *ap;
  const int lane = threadIdx.x & 31, nb = a.nb;
  const int j0 = 2 * lane, j1 = j0 + 1;
  const uint32_t c0 = j0 < nb ? a.counts[j0] : 0u, c1 = j1 < nb ? a.counts[j1] : 0u;
  // A list whose count exceeds its stride is one that overflowed its
  // threshold's capacity: it is incomplete, and refused.
  if (__any_sync(0xffffffffu, c0 > a.stride || c1 > a.stride)) {
    if (lane == 0)
      st->error |= kErrListOverflow;
    return;
  }
  uint32_t incl = c0 + c1;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o)
      incl += t;
  }
  const uint32_t excl = incl - c0 - c1;
  if (j0 < nb)
    st->frame_off[j0] = excl;
  if (j1 < nb)
    st->frame_off[j1] = excl + c0;
  const uint32_t off = __shfl_sync(0xffffffffu, incl, 31);
  if (lane != 0)
    return;
  st->frame_off[nb] = off;
  st->n_big = 0;
  st->n_edges = 0;
  const unsigned long long total = (unsigned long long)st->n_live + off;
  if (total > capacity) {
    st->error |= kErrLiveFull;
    return;
  }
  st->n_total = (uint32_t)total;
  st->counts[kCntSignal] += off;
}

// The batch's lists into the pool. Each warp appends 32 consecutive pixels
// and points each one straight at the first pixel of its run (consecutive
// indices of one row) within those 32: the union-find then starts from trees
// one level deep instead of chains along the rows, whose finds would walk
// the row at memory latency. Runs crossing a warp's boundary are joined by
// k_link's left-neighbour union.
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
  const uint32_t width = a.width;
  const sf_signal_pixel *list = lists + (size_t)j * stride;
  const int lane = threadIdx.x & 31;
  for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < n;
       i0 += gridDim.x * blockDim.x) {  // warp-uniform
    const uint32_t i = i0 + lane;
    const bool in = i < n;
    sf_signal_pixel s;
    s.index = 0;
    s.value = 0;
    if (in)
      s = list[i];
    const uint32_t before = __shfl_up_sync(0xffffffffu, s.index, 1);
    const bool starts = !in || lane == 0 || s.index % width == 0 || before != s.index - 1;
    const unsigned mask = __ballot_sync(0xffffffffu, starts) & (0xffffffffu >> (31 - lane));
    if (in) {
      const uint32_t p = base + i;
      frame[p] = a.frames[j];
      index[p] = s.index;
      value[p] = s.value;
      parent[p] = base + i0 + (31 - __clz(mask));
    }
  }
}

// Per-row start tables of the frames a batch links: segment 0 is the frame
// before the batch (the live pool's tail, [prev_start, n_live)), segment
// j + 1 the batch's frame j. rows[s * (height + 1) + y] is the first position
// of segment s whose index is at or beyond row y; entry `height` is the
// segment's end. Every entry is written once: by the pixel that starts the
// row (or the first pixel after a run of empty rows), or by the segment's
// last pixel for the rows after it.
__global__ void k_rows(LabelStatus *st, const BatchArgs *__restrict__ ap,
                       const uint32_t *__restrict__ index, uint32_t *__restrict__ rows,
                       uint32_t height) {
  if (st->error)
    return;
  const BatchArgs &a = *ap;
  const int s = blockIdx.y;
  uint32_t lo, hi;
  if (s == 0) {
    if (!a.link_prev[0])
      return;  // the batch's first frame does not link back: no table needed
    lo = st->prev_start;
    hi = st->n_live;
  } else {
    lo = st->n_live + st->frame_off[s - 1];
    hi = st->n_live + st->frame_off[s];
  }
  uint32_t *row = rows + (size_t)s * (height + 1);
  const uint32_t width = a.width;
  const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  if (lo == hi) {
    for (uint32_t y = t0; y <= height; y += nt)
      row[y] = lo;
    return;
  }
  for (uint32_t p = lo + t0; p < hi; p += nt) {
    const uint32_t y = index[p] / width;
    const uint32_t first = p == lo ? 0u : index[p - 1] / width + 1u;
    for (uint32_t r = first; r <= y; r++)
      row[r] = p;
    if (p == hi - 1)
      for (uint32_t r = y + 1; r <= height; r++)
        row[r] = hi;
  }
}

// Appends this lane's edges (p, q[k]) for the k with bit k of `want` set (at
// most three: left, above, previous frame) to the batch's edge list, with
// one atomic for the whole warp's edges; a lane whose edge finds the list
// full joins it at once.
__device__ __forceinline__ void push_edges(uint32_t want, uint32_t p, const uint32_t q[3],
                                           LabelStatus *st, uint2 *edges, uint32_t edge_cap,
                                           uint32_t *parent) {
  const int lane = threadIdx.x & 31;
  const uint32_t mine = (uint32_t)__popc(want);
  // The warp's inclusive prefix of edge counts.
  uint32_t inc = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o)
      inc += t;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
  if (total == 0)
    return;
  uint32_t base = 0;
  if (lane == 31)
    base = atomicAdd(&st->n_edges, total);
  base = __shfl_sync(0xffffffffu, base, 31);
  uint32_t at = base + inc - mine;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    if ((want >> k) & 1u) {
      if (at < edge_cap)
        edges[at] = make_uint2(p, q[k]);
      else
        uf_unite(parent, p, q[k], st);
      at++;
    }
  }
}

// dials_spots.cc:106-137: left (same row), above (same frame), and the same
// index on the previous frame when it is the one before. With row tables
// (rows non-null) the searches stay within one row of the list. The edges
// found go to a list that k_unite joins with every lane busy (here most lanes
// have none, and the joins' loops would run with a lane or two).
//
// Only the unions the others do not already imply are listed: k_append
// joined each run within its 32-pixel chunk, so the left link is needed only
// at a chunk's first pixel; and a pixel whose left neighbour (same run) has
// its own neighbour above (or on the previous frame) just left of this
// pixel's is joined through them -- those two are consecutive in their row,
// so in one run. Each overlap of two runs is listed once, at its first pixel.
// The components, and so the roots (lowest positions), are the same.
__global__ void k_link(LabelStatus *st, const BatchArgs *__restrict__ ap,
                       const uint32_t *__restrict__ index, uint32_t *parent,
                       const uint32_t *__restrict__ rows, uint32_t height, uint2 *edges,
                       uint32_t edge_cap) {
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
  const uint32_t *own = rows ? rows + (size_t)(j + 1) * (height + 1) : nullptr;
  const uint32_t *before = rows ? rows + (size_t)j * (height + 1) : nullptr;
  const int lane = threadIdx.x & 31;
  for (uint32_t p0 = start + blockIdx.x * blockDim.x + (threadIdx.x & ~31u); p0 < end;
       p0 += gridDim.x * blockDim.x) {  // warp-uniform
    const uint32_t p = p0 + lane;
    const bool in = p < end;
    const uint32_t idx = in ? index[p] : 0u;
    const uint32_t y = idx / width, x = idx - y * width;
    const bool left = in && p > start && x != 0 && index[p - 1] == idx - 1;
    uint32_t want = left && ((p - start) & 31u) == 0 ? 1u : 0u;
    uint32_t q[3] = {p - 1, 0u, 0u};
    {
      const uint32_t t = idx - width;
      uint32_t lo = 0, hi = 0;
      if (in && y > 0) {
        lo = own ? own[y - 1] : start;
        hi = own ? own[y] : p;
      }
      q[1] = lower_bound_warp(index, lo, hi, t);
      if (q[1] < hi && index[q[1]] == t && !(left && q[1] > lo && index[q[1] - 1] == t - 1))
        want |= 2u;
    }
    if (phi > plo) {  // uniform: the frame links back or not
      uint32_t lo = 0, hi = 0;
      if (in) {
        lo = before ? before[y] : plo;
        hi = before ? before[y + 1] : phi;
      }
      q[2] = lower_bound_warp(index, lo, hi, idx);
      if (q[2] < hi && index[q[2]] == idx &&
          !(left && q[2] > lo && index[q[2] - 1] == idx - 1))
        want |= 4u;
    }
    push_edges(want, p, q, st, edges, edge_cap, parent);
  }
}

// The listed edges joined, a thread each.
__global__ void k_unite(LabelStatus *st, const uint2 *__restrict__ edges, uint32_t edge_cap,
                        uint32_t *parent) {
  if (st->error)
    return;
  const uint32_t n = min(st->n_edges, edge_cap);
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += gridDim.x * blockDim.x) {
    const uint2 pq = edges[e];
    uf_unite(parent, pq.x, pq.y, st);
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
  const int lane = threadIdx.x & 31;
  // Whole warps walk the pool (the loop bound is warp-uniform); the lanes of
  // one component (consecutive pixels mostly share their root) add their
  // count and latest frame with one atomic each.
  for (uint32_t p0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); p0 < n;
       p0 += gridDim.x * blockDim.x) {
    const uint32_t p = p0 + lane;
    const bool in = p < n;
    const uint32_t r = in ? root[p] : kNone;
    const int32_t z = in ? frame[p] : INT_MIN;
    const unsigned same = __match_any_sync(0xffffffffu, r);
    const int32_t zmax = __reduce_max_sync(same, z);
    if (in && lane == __ffs(same) - 1) {
      atomicMax(&zlast[r], zmax);
      atomicAdd(&csize[r], (uint32_t)__popc(same));
    }
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

// This block's share [lo, hi) of n items (the histogram and the scatter
// split them alike).
__device__ __forceinline__ void bucket_chunk(uint32_t n, uint32_t *lo, uint32_t *hi) {
  const uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
  *lo = min(n, blockIdx.x * chunk);
  *hi = min(n, *lo + chunk);
}

__global__ void __launch_bounds__(kThreads)
k_bucket_hist(LabelStatus *st, const uint32_t *__restrict__ cbucket, uint32_t *hist) {
  if (st->error)
    return;
  __shared__ uint32_t h[kBuckets];
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
    h[b] = 0;
  __syncthreads();
  uint32_t lo, hi;
  bucket_chunk(st->n_closing, &lo, &hi);
  for (uint32_t k = lo + threadIdx.x; k < hi; k += blockDim.x)
    atomicAdd(&h[cbucket[k]], 1u);
  __syncthreads();
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
    hist[blockIdx.x * kBuckets + b] = h[b];
}

// Exclusive scan over (bucket, block) in bucket-major order, in place: a warp
// scans a bucket's counts (each lane a run of blocks), then the buckets'
// totals are scanned and added.
__global__ void __launch_bounds__(1024) k_bucket_offsets(LabelStatus *st, uint32_t *hist) {
  if (st->error)
    return;
  __shared__ uint32_t btotal[kBuckets];
  constexpr int kPer = (kGrid + 31) / 32;  // blocks a lane
  const int lane = threadIdx.x & 31;
  const int lo = min(kGrid, lane * kPer), hi = min(kGrid, lo + kPer);
  for (int b = threadIdx.x >> 5; b < kBuckets; b += blockDim.x >> 5) {  // warp-uniform
    uint32_t v[kPer], sum = 0;
#pragma unroll
    for (int k = 0; k < kPer; k++) {
      v[k] = lo + k < hi ? hist[(lo + k) * kBuckets + b] : 0u;
      sum += v[k];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o)
        incl += t;
    }
    uint32_t run = incl - sum;
#pragma unroll
    for (int k = 0; k < kPer; k++) {
      if (lo + k < hi)
        hist[(lo + k) * kBuckets + b] = run;
      run += v[k];
    }
    if (lane == 31)
      btotal[b] = incl;
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
  for (int i = threadIdx.x; i < kGrid * kBuckets; i += blockDim.x)
    hist[i] += btotal[i % kBuckets];
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
  bucket_chunk(st->n_closing, &lo, &hi);
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
  const int lane = threadIdx.x & 31;
  // The lanes of one candidate take their member slots with one atomic: a
  // run of slots whose positions ascend, from this warp's 32 positions,
  // which no other warp's run shares. The run's first slot is flagged
  // (kRunHead: positions are below 2^31, the pool's limit), so that k_sort
  // can order the runs instead of the members.
  for (uint32_t p0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); p0 < n;
       p0 += gridDim.x * blockDim.x) {
    const uint32_t p = p0 + lane;
    const uint32_t c = p < n ? candid[root[p]] : kNone;
    const unsigned same = __match_any_sync(0xffffffffu, c);
    const int leader = __ffs(same) - 1;
    uint32_t slot = 0;
    if (c != kNone && lane == leader)
      slot = atomicAdd(&cursor[c], (uint32_t)__popc(same));
    slot = __shfl_sync(0xffffffffu, slot, leader);
    if (c != kNone)
      members[cand_off[c] + slot + __popc(same & ((1u << lane) - 1u))] =
          p | (lane == leader ? kRunHead : 0u);
  }
}

// Bitonic sort of s[0 .. n) in shared memory by `nt` cooperating threads
// numbered t, ascending. Every comparator puts the smaller value first (each
// merge starts by comparing element i with its mirror in its block), so the
// length needs no padding: a comparator whose second element lies at or
// beyond n would leave the first in place, as if against +infinity, and is
// skipped. Threads walk the comparators, not the elements.
__device__ void bitonic_sort(uint32_t *s, int n, int t, int nt) {
  int size = 1;
  while (size < n)
    size <<= 1;
  for (int k = 2; k <= size; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      const int lj = __ffs(j) - 1;
      for (int q = t; q < (size >> 1); q += nt) {
        const int blk = q >> lj, r = q & (j - 1);
        int i, l;
        if (j == (k >> 1)) {
          i = blk * k + r;
          l = blk * k + k - 1 - r;
        } else {
          i = (blk << (lj + 1)) + r;
          l = i + j;
        }
        if (l < n) {
          const uint32_t x = s[i], y = s[l];
          if (x > y) {
            s[i] = y;
            s[l] = x;
          }
        }
      }
      __syncthreads();
    }
  }
}

// The same network for at most 32 values, one a lane, in registers: lane
// `lane` returns the lane-th smallest (values of lanes at or beyond n are
// +infinity).
__device__ __forceinline__ uint32_t warp_sort32(uint32_t v, int n, int lane) {
  if (lane >= n)
    v = kNone;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      // Partner: the mirror within the block of k at the merge's first step,
      // else the lane j away; the lower lane keeps the smaller value.
      const int partner = j == (k >> 1) ? (lane ^ (k - 1)) : (lane ^ j);
      const uint32_t o = __shfl_sync(0xffffffffu, v, partner);
      const bool low = lane < partner;
      v = low ? min(v, o) : max(v, o);
    }
  }
  return v;
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

__device__ __forceinline__ bool fp_finish(FirstPass &f) {
  const unsigned long long lim = 1ull << 53;
  f.exact = f.exact && f.S < lim && f.Q2 < lim && f.W[0] < lim && f.W[1] < lim && f.W[2] < lim;
  return f.exact;
}

// ---------------------------------------------------------------------------
// Emission (dials_spots.cc:221-360), arranged for GB300's FP64 rate (a small
// fraction of its integer rate: an FP64 instruction takes its issue slots on
// the FP64 pipe however few of its lanes are used). Every FP64 operation is
// the reference's, in its order; the work is laid out so that the lanes of
// each FP64 instruction are busy:
//
//   k_sort         a warp per candidate (a block beyond kWarpSortMax members
//                  or kWarpSegMax runs,
//                  a block sorting in global memory beyond kBlockSortMax):
//                  members sorted into (frame, index) order and copied out as
//                  pixel records, each tagged with its candidate.
//   k_first        a warp per candidate: the first pass as exact integer
//                  sums across the lanes (redux.sync); its FP64 part (the
//                  centroid divisions, the peak-separation test) then runs
//                  for 32 candidates at once, one a lane.
//   k_pix          a thread per member: the accepted spots' pixels out.
//   k_terms        a thread per member: its three variance-pass terms
//                  RN(RN(v d) d), d = (c + 0.5) - centre.
//   k_perm_*       the candidates ordered by size (largest first), so that
//                  the candidates sharing a warp in k_var have similar sizes.
//   k_var          four lanes per candidate, in size order: one axis a lane,
//                  the terms summed with rounding in member order (the one
//                  part whose order matters), the variances, the spot record.
//
// Where the integer sums could be inexact (a value of 2^26 or more, a
// coordinate beyond 2^20, sums beyond 2^53) the thread runs the reference's
// double sequence instead.
// ---------------------------------------------------------------------------

// What k_var needs of a candidate, from the first pass.
struct CandSpot {
  double pos[3];      // xyzobs (after the single-frame z and zero-sum rules)
  double cz;          // the z centroid before the single-frame rule: the variance pass's centre
  double sum, sum_sq; // intensity and the sum of squares
  int32_t bb[6];
  uint32_t n, mode;   // mode: kModeExact | kModeSpread
};
enum : uint32_t { kModeExact = 1u, kModeSpread = 2u };

// Members whose loads a thread keeps in flight in its sequential passes.
constexpr int kPipe = 8;

// x = index mod width, y = index / width by the batch's multiply-high
// divisor (Granlund & Montgomery's round-up method, exact for every 32-bit
// index and width).
__device__ __forceinline__ void pixel_xyz(const sf_pixel &px, const BatchArgs &a, int32_t *x,
                                          int32_t *y, int32_t *z) {
  const uint32_t t = __umulhi(px.index, a.wdiv_m);
  const uint32_t y0 = (t + ((px.index - t) >> a.wdiv_s1)) >> a.wdiv_s2;
  *x = (int32_t)(px.index - y0 * a.width);
  *y = (int32_t)y0;
  *z = px.frame;
}

// c + 0.5 as a double for an integer 0 <= c < 2^30, built from the bits of
// 2c + 1 (exactly the value (double)c + 0.5 rounds to, with no FP64 work).
__device__ __forceinline__ double half_up(uint32_t c) {
  const uint32_t u = 2u * c + 1u;
  const int e = 31 - __clz(u);
  const unsigned long long m = ((unsigned long long)u << (52 - e)) & ((1ull << 52) - 1ull);
  return __longlong_as_double(((unsigned long long)(1022 + e) << 52) | m);
}

// (double)v for an unsigned 32-bit v, from its bits.
__device__ __forceinline__ double exact_double(uint32_t v) {
  if (v == 0)
    return 0.0;
  const int e = 31 - __clz(v);
  const unsigned long long m = ((unsigned long long)v << (52 - e)) & ((1ull << 52) - 1ull);
  return __longlong_as_double(((unsigned long long)(1023 + e) << 52) | m);
}

// The FP64 part of the first pass of emit() and the peak-separation test
// (dials_spots.cc:240-330) for one candidate whose members mp[0 .. n) are in
// member order: from the exact integer sums f when f.exact, else the
// reference's double sequence over the members. Fills *out and returns
// acceptance.
__device__ bool accept_candidate(const sf_pixel *mp, uint32_t n, const BatchArgs &a,
                                 const FirstPass &f, CandSpot *out) {
  CandSpot c;
  double weighted[3], peak[3] = {0.0, 0.0, 0.0};
  if (f.exact) {
    c.sum = (double)f.S;
    c.sum_sq = (double)f.Q2;
    for (int ax = 0; ax < 3; ax++)
      weighted[ax] = __dmul_rn((double)f.W[ax], 0.5);  // exact: W < 2^53
    if (f.peak_k != 0xFFFFFFFFu) {
      int32_t px, py, pz;
      pixel_xyz(mp[f.peak_k], a, &px, &py, &pz);
      peak[0] = __dadd_rn((double)px, 0.5);
      peak[1] = __dadd_rn((double)py, 0.5);
      peak[2] = __dadd_rn((double)pz, 0.5);
    }
  } else {
    c.sum = c.sum_sq = 0.0;
    weighted[0] = weighted[1] = weighted[2] = 0.0;
    uint32_t peak_value = 0;
    for (uint32_t k = 0; k < n; k++) {
      int32_t x, y, z;
      pixel_xyz(mp[k], a, &x, &y, &z);
      const uint32_t v = mp[k].value;
      const double val = (double)v;
      const double pos[3] = {__dadd_rn((double)x, 0.5), __dadd_rn((double)y, 0.5),
                             __dadd_rn((double)z, 0.5)};
      c.sum = __dadd_rn(c.sum, val);
      c.sum_sq = __dadd_rn(c.sum_sq, __dmul_rn(val, val));
      for (int ax = 0; ax < 3; ax++)
        weighted[ax] = __dadd_rn(weighted[ax], __dmul_rn(val, pos[ax]));
      if (v > peak_value) {
        peak_value = v;
        peak[0] = pos[0], peak[1] = pos[1], peak[2] = pos[2];
      }
    }
  }
  for (int b = 0; b < 6; b++)
    c.bb[b] = f.bb[b];
  c.n = n;
  c.mode = (f.exact ? kModeExact : 0u) | (c.sum > 0.0 ? kModeSpread : 0u);
  if (c.sum > 0.0) {
    for (int ax = 0; ax < 3; ax++)
      c.pos[ax] = __ddiv_rn(weighted[ax], c.sum);
    c.cz = c.pos[2];
    if (c.bb[5] == c.bb[4] + 1)
      c.pos[2] = __dadd_rn((double)c.bb[4], 0.5);
  } else {
    c.pos[0] = __ddiv_rn((double)(c.bb[1] + c.bb[0]), 2.0);
    c.pos[1] = __ddiv_rn((double)(c.bb[3] + c.bb[2]), 2.0);
    c.pos[2] = __ddiv_rn((double)(c.bb[5] + c.bb[4]), 2.0);
    c.cz = c.pos[2];
  }
  *out = c;
  if (a.max_separation > 0.0) {
    const double dx = __dsub_rn(peak[0], c.pos[0]);
    const double dy = __dsub_rn(peak[1], c.pos[1]);
    const double dz = __dsub_rn(peak[2], c.pos[2]);
    const double d2 =
        __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (__dsqrt_rn(d2) > a.max_separation)
      return false;
  }
  return true;
}

// Member k (in member order) of candidate c: its pixel record and tag.
__device__ __forceinline__ void put_member(uint32_t q, uint32_t k, uint32_t c, uint32_t off,
                                           const int32_t *__restrict__ frame,
                                           const uint32_t *__restrict__ index,
                                           const uint32_t *__restrict__ value, sf_pixel *mpix,
                                           uint32_t *mcand) {
  sf_pixel px;
  px.frame = frame[q];
  px.index = index[q];
  px.value = value[q];
  mpix[off + k] = px;
  mcand[off + k] = c;
}

// Member positions put in ascending order, then copied out in member order
// as pixel records. A warp each (BLOCK false): a candidate of up to 32
// members is sorted in registers; one of up to kWarpSortMax members in at
// most kWarpSegMax runs (k_gather's runs of ascending positions, each from
// its own range of positions) is ordered by its runs: a run's place is the
// total length of the runs whose first position is smaller. The others, up
// to kBlockSortMax members, go on a list for a block each (BLOCK true),
// which sorts them in shared memory (bitonic).
template <bool BLOCK>
__global__ void __launch_bounds__(kThreads)
k_sort(LabelStatus *st, const uint32_t *__restrict__ cand_n,
       const uint32_t *__restrict__ cand_off, const uint32_t *__restrict__ members,
       const int32_t *__restrict__ frame, const uint32_t *__restrict__ index,
       const uint32_t *__restrict__ value, sf_pixel *mpix, uint32_t *mcand, uint32_t *big) {
  if (st->error)
    return;
  extern __shared__ __align__(16) uint32_t s_sort[];
  const uint32_t ncand = st->n_cand;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  if (!BLOCK) {
    uint32_t *s = s_sort + warp * (kWarpSortMax + 2 * kWarpSegMax);
    uint32_t *seg = s + kWarpSortMax;  // runs: first slots, then first positions / places
    for (uint32_t c = blockIdx.x * nwarps + warp; c < ncand; c += gridDim.x * nwarps) {
      const uint32_t n = cand_n[c];
      if (n > (uint32_t)kWarpSortMax) {
        if (lane == 0)
          big[atomicAdd(&st->n_big, 1u)] = c;  // for the block sorts, in any order
        continue;
      }
      const uint32_t off = cand_off[c];
      const uint32_t *m = members + off;
      if (n <= 32) {
        const uint32_t q =
            warp_sort32(lane < (int)n ? m[lane] & kPosMask : kNone, (int)n, lane);
        if (lane < (int)n)
          put_member(q, lane, c, off, frame, index, value, mpix, mcand);
        continue;
      }
      // The slots into shared memory (flags kept), the runs' first slots and
      // positions noted.
      uint32_t nrun = 0;
      for (uint32_t b = 0; b < n; b += 32) {  // warp-uniform
        const uint32_t i = b + lane;
        const uint32_t x = i < n ? m[i] : 0u;
        const bool head = (x & kRunHead) != 0u;
        if (i < n)
          s[i] = x;
        const unsigned bal = __ballot_sync(0xffffffffu, head);
        const uint32_t k = nrun + (uint32_t)__popc(bal & ((1u << lane) - 1u));
        if (head && k < (uint32_t)kWarpSegMax) {
          seg[k] = i;
          seg[kWarpSegMax + k] = x & kPosMask;
        }
        nrun += (uint32_t)__popc(bal);
      }
      __syncwarp();
      if (nrun <= (uint32_t)kWarpSegMax && seg[0] == 0u) {  // slot 0 always heads a run
        // A lane's runs j = lane + 32 h: their first positions, then the
        // total length of the runs whose first position is smaller.
        const int hn = (int)((nrun + 31u) >> 5);  // a lane's runs in use (warp-uniform)
        uint32_t first[kSegPerLane], place[kSegPerLane];
#pragma unroll
        for (int h = 0; h < kSegPerLane; h++) {
          const uint32_t j = (uint32_t)lane + 32u * h;
          first[h] = j < nrun ? seg[kWarpSegMax + j] : kNone;
          place[h] = 0u;
        }
        for (uint32_t t = 0; t < nrun; t++) {  // warp-uniform
          const uint32_t ft = seg[kWarpSegMax + t];
          const uint32_t lt = (t + 1 < nrun ? seg[t + 1] : n) - seg[t];
#pragma unroll
          for (int h = 0; h < kSegPerLane; h++)
            if (h < hn)
              place[h] += ft < first[h] ? lt : 0u;
        }
        __syncwarp();
#pragma unroll
        for (int h = 0; h < kSegPerLane; h++) {
          const uint32_t j = (uint32_t)lane + 32u * h;
          if (j < nrun)
            seg[kWarpSegMax + j] = place[h];
        }
        __syncwarp();
        uint32_t runs = 0;
        for (uint32_t b = 0; b < n; b += 32) {  // warp-uniform
          const uint32_t i = b + lane;
          const uint32_t x = i < n ? s[i] : 0u;
          const unsigned bal = __ballot_sync(0xffffffffu, (x & kRunHead) != 0u);
          // The run of slot i: the last head at or before it.
          const uint32_t g = runs + (uint32_t)__popc(bal & ((2u << lane) - 1u)) - 1u;
          runs += (uint32_t)__popc(bal);
          if (i < n)
            put_member(x & kPosMask, seg[kWarpSegMax + g] + (i - seg[g]), c, off, frame, index,
                       value, mpix, mcand);
        }
        __syncwarp();  // the next candidate reuses the shared rows
        continue;
      }
      // More runs than a warp orders: a block sorts the members (a warp's
      // sort of a few hundred members would hold up its SM's last wave).
      if (lane == 0)
        big[atomicAdd(&st->n_big, 1u)] = c;
      __syncwarp();  // the next candidate reuses the shared rows
    }
  } else {
    const uint32_t nbig = st->n_big;
    for (uint32_t b = blockIdx.x; b < nbig; b += gridDim.x) {
      const uint32_t c = big[b];
      const uint32_t n = cand_n[c];
      if (n > (uint32_t)kBlockSortMax)
        continue;
      const uint32_t off = cand_off[c];
      const uint32_t *m = members + off;
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        s_sort[i] = m[i] & kPosMask;
      __syncthreads();
      bitonic_sort(s_sort, (int)n, threadIdx.x, blockDim.x);
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        put_member(s_sort[i], i, c, off, frame, index, value, mpix, mcand);
      __syncthreads();
    }
  }
}

// Candidates beyond kBlockSortMax members (possible when max_spot_size allows
// them): a block each sorts the member positions in place in global memory
// with a bitonic network whose every comparator puts the smaller value first
// (each merge starts by comparing element i with its mirror in the block), so
// the length needs no padding -- a comparator whose second element lies
// beyond the end would leave the first in place, as if against +infinity.
__global__ void __launch_bounds__(kThreads)
k_sort_big(LabelStatus *st, const uint32_t *__restrict__ cand_n,
           const uint32_t *__restrict__ cand_off, uint32_t *members,
           const int32_t *__restrict__ frame, const uint32_t *__restrict__ index,
           const uint32_t *__restrict__ value, sf_pixel *mpix, uint32_t *mcand,
           const uint32_t *__restrict__ big) {
  if (st->error)
    return;
  const uint32_t nbig = st->n_big;
  for (uint32_t b = blockIdx.x; b < nbig; b += gridDim.x) {
    const uint32_t c = big[b];
    const uint32_t n = cand_n[c];
    if (n <= (uint32_t)kBlockSortMax)
      continue;
    const uint32_t off = cand_off[c];
    uint32_t *m = members + off;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
      m[i] &= kPosMask;  // the run flags (k_gather)
    __syncthreads();
    uint32_t size = 1;
    while (size < n)
      size <<= 1;
    for (uint32_t k = 2; k <= size; k <<= 1) {
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        for (uint32_t t = threadIdx.x; t < size / 2; t += blockDim.x) {
          const uint32_t blk = t / j, r = t - blk * j;
          uint32_t i, l;
          if (j == (k >> 1)) {  // the mirror comparator of the merge's first step
            i = blk * k + r;
            l = blk * k + k - 1 - r;
          } else {
            i = blk * 2 * j + r;
            l = i + j;
          }
          if (l < n) {
            const uint32_t x = m[i], y = m[l];
            if (x > y) {
              m[i] = y;
              m[l] = x;
            }
          }
        }
        __syncthreads();
      }
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
      put_member(m[i], i, c, off, frame, index, value, mpix, mcand);
    __syncthreads();
  }
}

// The candidates ordered by size, largest first (a counting sort over
// kSizeBins bins; sizes of kSizeBins - 1 and more share the first bin, and
// the order within a bin is arbitrary): perm[i] is the i-th candidate to
// process. hist holds 2 * kSizeBins words.
constexpr int kSizeBins = 1024;

__device__ __forceinline__ uint32_t size_bin(uint32_t n) {
  return (uint32_t)(kSizeBins - 1) - min(n, (uint32_t)(kSizeBins - 1));
}

__global__ void k_perm_hist(LabelStatus *st, const uint32_t *__restrict__ cand_n,
                            uint32_t *hist) {
  if (st->error)
    return;
  __shared__ uint32_t h[kSizeBins];
  for (int b = threadIdx.x; b < kSizeBins; b += blockDim.x)
    h[b] = 0;
  __syncthreads();
  const uint32_t ncand = st->n_cand;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncand;
       c += gridDim.x * blockDim.x)
    atomicAdd(&h[size_bin(cand_n[c])], 1u);
  __syncthreads();
  for (int b = threadIdx.x; b < kSizeBins; b += blockDim.x)
    if (h[b])
      atomicAdd(&hist[b], h[b]);
}

// One block: the bins' exclusive offsets (into the cursors, hist +
// kSizeBins), and the counts cleared for the next call.
__global__ void __launch_bounds__(kSizeBins) k_perm_offsets(LabelStatus *st, uint32_t *hist) {
  if (st->error)
    return;
  uint32_t total;
  const uint32_t v = hist[threadIdx.x];
  const uint32_t e = block_exclusive_scan(v, &total);
  hist[kSizeBins + threadIdx.x] = e;
  hist[threadIdx.x] = 0;
}

__global__ void k_perm_scatter(LabelStatus *st, const uint32_t *__restrict__ cand_n,
                               uint32_t *hist, uint32_t *perm) {
  if (st->error)
    return;
  const uint32_t ncand = st->n_cand;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncand;
       c += gridDim.x * blockDim.x)
    perm[atomicAdd(&hist[kSizeBins + size_bin(cand_n[c])], 1u)] = c;
}

// Warp-wide sum modulo 2^64 of one 64-bit value a lane, by redux.sync on
// 22-bit limbs (each limb's sum over 32 lanes fits in 32 bits).
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
  const uint32_t l0 = (uint32_t)v & 0x3FFFFFu, l1 = (uint32_t)(v >> 22) & 0x3FFFFFu,
                 l2 = (uint32_t)(v >> 44);
  return (unsigned long long)__reduce_add_sync(0xffffffffu, l0) +
         ((unsigned long long)__reduce_add_sync(0xffffffffu, l1) << 22) +
         ((unsigned long long)__reduce_add_sync(0xffffffffu, l2) << 44);
}

// A warp per candidate: the first pass (exact integer sums, dials_spots.cc:
// 240-276) over the members, a lane every 32nd, reduced across the warp. The
// finished first passes wait, one a lane, until 32 are ready; then their FP64
// part (acceptance) runs for 32 candidates at once, every lane busy.
__global__ void __launch_bounds__(kThreads)
k_first(LabelStatus *st, const BatchArgs *__restrict__ ap, const uint32_t *__restrict__ cand_n,
        const uint32_t *__restrict__ cand_off, const sf_pixel *__restrict__ mpix, CandSpot *cs,
        uint32_t *acc, uint32_t *acc_n) {
  const BatchArgs &a = *ap;
  if (st->error)
    return;
  const uint32_t ncand = st->n_cand;
  const int lane = threadIdx.x & 31;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  FirstPass held;
  fp_init(held);
  uint32_t held_c = 0, held_n = 0, separated = 0;
  int nheld = 0;
  auto flush = [&]() {
    if (lane < nheld) {
      CandSpot spot;
      const bool ok = accept_candidate(mpix + cand_off[held_c], held_n, a, held, &spot);
      cs[held_c] = spot;
      acc[held_c] = ok ? 1u : 0u;
      acc_n[held_c] = ok ? held_n : 0u;
      separated += ok ? 0u : 1u;
    }
    nheld = 0;
  };
  for (uint32_t c = gw; c < ncand; c += nw) {
    const uint32_t n = cand_n[c];
    const sf_pixel *mp = mpix + cand_off[c];
    FirstPass f;
    fp_init(f);
    for (uint32_t k = lane; k < n; k += 32) {
      int32_t x, y, z;
      const sf_pixel px = mp[k];
      pixel_xyz(px, a, &x, &y, &z);
      fp_add(f, k, px.value, x, y, z);
    }
    FirstPass g;
    g.S = warp_sum_u64(f.S);
    g.Q2 = warp_sum_u64(f.Q2);
    for (int ax = 0; ax < 3; ax++)
      g.W[ax] = warp_sum_u64(f.W[ax]);
    for (int b = 0; b < 6; b += 2) {
      g.bb[b] = __reduce_min_sync(0xffffffffu, f.bb[b]);
      g.bb[b + 1] = __reduce_max_sync(0xffffffffu, f.bb[b + 1]);
    }
    // The brightest value, and the first member holding it.
    const bool has = f.peak_k != 0xFFFFFFFFu;
    g.peak_v = __reduce_max_sync(0xffffffffu, has ? f.peak_v : 0u);
    g.peak_k = __reduce_min_sync(0xffffffffu,
                                 has && g.peak_v > 0 && f.peak_v == g.peak_v ? f.peak_k
                                                                             : 0xFFFFFFFFu);
    g.exact = __all_sync(0xffffffffu, f.exact) != 0;
    fp_finish(g);
    if (lane == nheld) {
      held = g;
      held_c = c;
      held_n = n;
    }
    if (++nheld == 32)
      flush();
  }
  if (nheld)
    flush();
  separated = __reduce_add_sync(0xffffffffu, separated);
  if (lane == 0 && separated)
    atomicAdd(&st->counts[kCntSeparated], (unsigned long long)separated);
}

// A thread per member of the batch's candidates whose sums are exact and
// positive: the member's three variance-pass terms RN(RN(v d) d), d =
// (c + 0.5) - centre (dials_spots.cc:331-341), every lane busy. c + 0.5 and
// v are built as doubles from their bits (coordinates below 2^20, values
// below 2^26 there).
__global__ void k_terms(LabelStatus *st, const BatchArgs *__restrict__ ap,
                        const sf_pixel *__restrict__ mpix, const uint32_t *__restrict__ mcand,
                        const uint32_t *__restrict__ acc, const CandSpot *__restrict__ cs,
                        double *__restrict__ terms, size_t terms_stride) {
  const BatchArgs &a = *ap;
  if (st->error)
    return;
  const uint32_t n = st->n_cand_pixels;
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < n;
       m += gridDim.x * blockDim.x) {
    const uint32_t c = mcand[m];
    if (!acc[c] || (cs[c].mode & (kModeExact | kModeSpread)) != (kModeExact | kModeSpread))
      continue;
    const sf_pixel px = mpix[m];
    int32_t coord[3];
    pixel_xyz(px, a, &coord[0], &coord[1], &coord[2]);
    const double centre[3] = {cs[c].pos[0], cs[c].pos[1], cs[c].cz};
    const double val = exact_double(px.value);
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
      const double d = __dsub_rn(half_up((uint32_t)coord[ax]), centre[ax]);
      terms[ax * terms_stride + m] = __dmul_rn(__dmul_rn(val, d), d);
    }
  }
}

// A thread per member of the batch's candidates: the accepted spots' pixels
// into the batch output, in member order (dials_spots.cc:355-359).
__global__ void k_pix(LabelStatus *st, const sf_pixel *__restrict__ mpix,
                      const uint32_t *__restrict__ mcand, const uint32_t *__restrict__ cand_off,
                      const uint32_t *__restrict__ acc, const uint32_t *__restrict__ acc_off,
                      sf_pixel *pixels, size_t pixels_cap) {
  if (st->error)
    return;
  const uint32_t n = st->n_cand_pixels;
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < n;
       m += gridDim.x * blockDim.x) {
    const uint32_t c = mcand[m];
    if (!acc[c])
      continue;
    const size_t at = (size_t)acc_off[c] + (m - cand_off[c]);
    if (at >= pixels_cap) {
      atomicOr(&st->error, kErrOutFull);
      continue;
    }
    pixels[at] = mpix[m];
  }
}

// The reference's variance pass (dials_spots.cc:331-353) over members in
// order, in double, as it writes it.
__device__ void variance_sequence(const sf_pixel *mp, uint32_t n, const BatchArgs &a,
                                  const double centre[3], double delta_sq[3]) {
  delta_sq[0] = delta_sq[1] = delta_sq[2] = 0.0;
  for (uint32_t k = 0; k < n; k++) {
    int32_t coord[3];
    pixel_xyz(mp[k], a, &coord[0], &coord[1], &coord[2]);
    const double val = (double)mp[k].value;
    for (int ax = 0; ax < 3; ax++) {
      const double d = __dsub_rn(__dadd_rn((double)coord[ax], 0.5), centre[ax]);
      delta_sq[ax] = __dadd_rn(delta_sq[ax], __dmul_rn(__dmul_rn(val, d), d));
    }
  }
}

// Four lanes per candidate, in size order (so that the candidates sharing a
// warp have similar sizes): lanes 0-2 each run one axis of the variance pass
// -- the reference's rounded additions of the member terms, in member order
// (dials_spots.cc:331-353) -- and the variance formula; lane 0 writes the
// accepted spot's record. Where the first pass was not exact, lane 0 runs the
// whole sequence alone.
__global__ void k_var(LabelStatus *st, const BatchArgs *__restrict__ ap,
                      const uint32_t *__restrict__ perm, const uint32_t *__restrict__ cand_off,
                      const uint32_t *__restrict__ acc, const uint32_t *__restrict__ acc_idx,
                      const uint32_t *__restrict__ acc_off, const CandSpot *__restrict__ cs,
                      const sf_pixel *__restrict__ mpix, const double *__restrict__ terms,
                      size_t terms_stride, sf_spot *spots, size_t spots_cap) {
  const BatchArgs &a = *ap;
  if (st->error)
    return;
  const uint32_t ncand = st->n_cand;
  const int sub = threadIdx.x & 3;
  const uint32_t per_pass = (gridDim.x * blockDim.x) >> 2;
  for (uint32_t base = (blockIdx.x * blockDim.x) >> 2; base < ncand; base += per_pass) {
    const uint32_t i = base + (threadIdx.x >> 2);
    const uint32_t c = i < ncand ? perm[i] : 0u;
    const bool live = i < ncand && acc[c];
    double var_ax = 0.0;
    CandSpot cd;
    if (live) {
      cd = cs[c];
      const uint32_t off = cand_off[c];
      if ((cd.mode & (kModeExact | kModeSpread)) == (kModeExact | kModeSpread) && sub < 3) {
        const double *t = terms + sub * terms_stride + off;
        double sum = 0.0;
        uint32_t k = 0;
        for (; k + kPipe <= cd.n; k += kPipe) {
          double x[kPipe];
#pragma unroll
          for (int u = 0; u < kPipe; u++)
            x[u] = t[k + u];
#pragma unroll
          for (int u = 0; u < kPipe; u++)
            sum = __dadd_rn(sum, x[u]);
        }
        for (; k < cd.n; k++)
          sum = __dadd_rn(sum, t[k]);
        const double ss = __dmul_rn(cd.sum, cd.sum);
        var_ax = ss > cd.sum_sq
                     ? __dadd_rn(__ddiv_rn(__ddiv_rn(__dmul_rn(sum, cd.sum),
                                                     __dsub_rn(ss, cd.sum_sq)),
                                           cd.sum),
                                 1.0 / 12.0)
                     : 1.0 / 12.0;
      }
    }
    const double v1 = __shfl_down_sync(0xffffffffu, var_ax, 1);
    const double v2 = __shfl_down_sync(0xffffffffu, var_ax, 2);
    if (!live || sub != 0)
      continue;
    const uint32_t si = acc_idx[c];
    if (si >= spots_cap) {
      atomicOr(&st->error, kErrOutFull);
      continue;
    }
    sf_spot spot;
    for (int b = 0; b < 6; b++)
      spot.bbox[b] = cd.bb[b];
    spot.position[0] = cd.pos[0];
    spot.position[1] = cd.pos[1];
    spot.position[2] = cd.pos[2];
    spot.intensity = cd.sum;
    spot.intensity_variance = cd.sum;
    spot.n_signal = cd.n;
    spot.variance[0] = spot.variance[1] = spot.variance[2] = 0.0;
    if (cd.mode & kModeSpread) {
      if (cd.mode & kModeExact) {
        spot.variance[0] = var_ax;
        spot.variance[1] = v1;
        spot.variance[2] = v2;
      } else {
        double delta_sq[3];
        const double centre[3] = {cd.pos[0], cd.pos[1], cd.cz};
        variance_sequence(mpix + cand_off[c], cd.n, a, centre, delta_sq);
        const double ss = __dmul_rn(cd.sum, cd.sum);
        for (int ax = 0; ax < 3; ax++)
          spot.variance[ax] =
              ss > cd.sum_sq
                  ? __dadd_rn(__ddiv_rn(__ddiv_rn(__dmul_rn(delta_sq[ax], cd.sum),
                                                  __dsub_rn(ss, cd.sum_sq)),
                                        cd.sum),
                              1.0 / 12.0)
                  : 1.0 / 12.0;
      }
    }
    spot.first = a.pixel_base + acc_off[c];
    spots[si] = spot;
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
  // A caller's say over growth (the served form's memory budget): asked for
  // the bytes of each new chunk before it is allocated; a refusal leaves the
  // store as it is and sets `refused`.
  LabelGrowth growth{};
  bool refused = false;
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
      if (growth.ok && !growth.ok(growth.ctx, c * sizeof(T))) {
        refused = true;
        return cudaErrorMemoryAllocation;
      }
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

// Every kernel of a label call loaded on the current device (a no-op once
// they are), by asking for each one's attributes.
static cudaError_t load_label_kernels() {
  const void *kernels[] = {
      (const void *)k_offsets,        (const void *)k_append,        (const void *)k_rows,
      (const void *)k_link,           (const void *)k_unite,         (const void *)k_flatten,
      (const void *)k_comp_stats,     (const void *)k_closing_flags, (const void *)k_closing_list,
      (const void *)k_bucket_hist,    (const void *)k_bucket_offsets,
      (const void *)k_bucket_scatter, (const void *)k_size_filter,   (const void *)k_cand_list,
      (const void *)k_gather,         (const void *)k_sort<false>,   (const void *)k_sort<true>,
      (const void *)k_sort_big,       (const void *)k_perm_hist,     (const void *)k_perm_offsets,
      (const void *)k_perm_scatter,   (const void *)k_first,         (const void *)k_pix,
      (const void *)k_terms,          (const void *)k_var,           (const void *)k_compact,
      (const void *)k_end_batch,      (const void *)scan_sums,       (const void *)scan_apply};
  for (const void *k : kernels) {
    cudaFuncAttributes a;
    const cudaError_t e = cudaFuncGetAttributes(&a, k);
    if (e != cudaSuccess)
      return e;
  }
  return cudaSuccess;
}

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
  // Per-row start tables (frames of at most kRowTableMaxRows rows), the
  // candidates' members as pixel records in member order with their
  // candidate, the candidates' first passes, and the variance terms.
  uint32_t *rows = nullptr, *mcand = nullptr, *big = nullptr, *perm = nullptr, *phist = nullptr;
  sf_pixel *mpix = nullptr;
  CandSpot *cspots = nullptr;
  double *terms = nullptr;
  uint2 *edges = nullptr;  // the unions k_link lists, capacity of them
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
  // With blocking waits (label_set_blocking_wait), a call's end is waited
  // for on this event, created with cudaEventBlockingSync: the calling thread
  // sleeps instead of spinning (the served form runs a thread per sweep).
  cudaEvent_t call_done = nullptr;
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
    cudaFree(rows);
    cudaFree(mcand);
    cudaFree(big);
    cudaFree(mpix);
    cudaFree(cspots);
    cudaFree(perm);
    cudaFree(phist);
    cudaFree(terms);
    cudaFree(edges);
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
    if (call_done)
      cudaEventDestroy(call_done);
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
    // At most one accepted spot (and one candidate) per min_spot_size pixels
    // closed in a batch.
    spots_cap = n / (opt.min_spot_size ? opt.min_spot_size : 1) + 1;
    if (height <= kRowTableMaxRows)
      SF_ALLOC(rows, (size_t)(kLabelMaxBatch + 1) * (height + 1));
    SF_ALLOC(mcand, n);
    // Every candidate a block sorts has more than 32 members (fewer are
    // sorted in a warp's registers).
    SF_ALLOC(big, n / 33 + 1);
    SF_ALLOC(mpix, n);
    SF_ALLOC(cspots, spots_cap);
    SF_ALLOC(perm, spots_cap);
    SF_ALLOC(phist, 2 * kSizeBins);
    SF_ALLOC(terms, 3 * n);
    SF_ALLOC(edges, n);
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
    if ((e = cudaMemsetAsync(st, 0, sizeof(LabelStatus), own_stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(phist, 0, 2 * kSizeBins * sizeof(uint32_t), own_stream)) !=
            cudaSuccess)
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
    if (rows)
      k_rows<<<dim3(kGrid / 4 > 0 ? kGrid / 4 : 1, nb + 1), kThreads, 0, s>>>(
          st, ap, index[c], rows, (uint32_t)height);
    k_link<<<g2, kThreads, 0, s>>>(st, ap, index[c], parent[c], rows, (uint32_t)height, edges,
                                   (uint32_t)capacity);
    k_unite<<<kPassGrid, kThreads, 0, s>>>(st, edges, (uint32_t)capacity, parent[c]);
    k_flatten<<<kPassGrid, kThreads, 0, s>>>(st, parent[c], root, zlast, csize, candid);
    k_comp_stats<<<kPassGrid, kThreads, 0, s>>>(st, root, frame[c], zlast, csize);
    k_closing_flags<<<kPassGrid, kThreads, 0, s>>>(st, ap, root, zlast, flag, open);
    const uint32_t *err = &st->error;
    if ((e = exclusive_scan(flag, posa, &st->n_total, &st->n_closing, block_sums, err, s)) !=
        cudaSuccess)
      return e;
    k_closing_list<<<kPassGrid, kThreads, 0, s>>>(st, ap, flag, posa, zlast, clist, cbucket);
    k_bucket_hist<<<kGrid, kThreads, 0, s>>>(st, cbucket, hist);
    k_bucket_offsets<<<1, 1024, 0, s>>>(st, hist);
    k_bucket_scatter<<<kGrid, kThreads, 0, s>>>(st, clist, cbucket, hist, order);
    k_size_filter<<<kPassGrid, kThreads, 0, s>>>(st, ap, order, csize, cflag);
    if ((e = exclusive_scan(cflag, cpos, &st->n_closing, &st->n_cand, block_sums, err, s)) !=
        cudaSuccess)
      return e;
    k_cand_list<<<kPassGrid, kThreads, 0, s>>>(st, order, csize, cflag, cpos, cand_root, cand_n,
                                           candid, cursor);
    if ((e = exclusive_scan(cand_n, cand_off, &st->n_cand, &st->n_cand_pixels, block_sums,
                            err, s)) != cudaSuccess)
      return e;
    k_gather<<<kPassGrid, kThreads, 0, s>>>(st, root, candid, cand_off, cursor, members);
    k_sort<false><<<kSortGrid, kThreads,
                    (kThreads / 32) * (kWarpSortMax + 2 * kWarpSegMax) * 4, s>>>(
        st, cand_n, cand_off, members, frame[c], index[c], value[c], mpix, mcand, big);
    k_sort<true><<<kGrid / 2, kThreads, kBlockSortMax * 4, s>>>(
        st, cand_n, cand_off, members, frame[c], index[c], value[c], mpix, mcand, big);
    k_sort_big<<<kGrid / 8, kThreads, 0, s>>>(st, cand_n, cand_off, members, frame[c],
                                              index[c], value[c], mpix, mcand, big);
    k_perm_hist<<<kGrid, kThreads, 0, s>>>(st, cand_n, phist);
    k_perm_offsets<<<1, kSizeBins, 0, s>>>(st, phist);
    k_perm_scatter<<<kPassGrid, kThreads, 0, s>>>(st, cand_n, phist, perm);
    k_first<<<kPassGrid, kThreads, 0, s>>>(st, ap, cand_n, cand_off, mpix, cspots, acc, acc_n);
    if ((e = exclusive_scan(acc, acc_idx, &st->n_cand, &st->n_accept, block_sums, err, s)) !=
        cudaSuccess)
      return e;
    if ((e = exclusive_scan(acc_n, acc_off, &st->n_cand, &st->n_accept_pixels, block_sums,
                            err, s)) != cudaSuccess)
      return e;
    k_pix<<<kPassGrid, kThreads, 0, s>>>(st, mpix, mcand, cand_off, acc, acc_off, d_pixels,
                                         capacity);
    k_terms<<<kPassGrid, kThreads, 0, s>>>(st, ap, mpix, mcand, acc, cspots, terms, capacity);
    k_var<<<kPassGrid, kThreads, 0, s>>>(st, ap, perm, cand_off, acc, acc_idx, acc_off, cspots,
                                         mpix, terms, capacity, d_spots, spots_cap);
    if ((e = exclusive_scan(open, posb, &st->n_total, &st->n_open, block_sums, err, s)) !=
        cudaSuccess)
      return e;
    k_compact<<<kPassGrid, kThreads, 0, s>>>(st, open, posb, root, frame[c], index[c], value[c],
                                         frame[o], index[o], value[o], parent[o]);
    k_end_batch<<<1, 32, 0, s>>>(st, ap);
    return cudaGetLastError();
  }

  // The sequence for (nb, c) as a CUDA graph, captured on the labeller's own
  // stream the second time that shape is met (the first runs directly, so
  // every kernel is loaded before a capture), then replayed on any stream.
  // Null if capture is not possible (the caller's stream is itself being
  // captured, or the capture failed): the sequence then runs directly.
  cudaGraphExec_t graph_for(int nb, int c, cudaStream_t s, bool now = false) {
    cudaGraphExec_t &g = graphs[c][nb];
    if (g || !use_graphs)
      return g;
    if (!seen[c][nb] && !now) {
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

  // Every batch size up to max_nb captured now, on both live pools, so that
  // no later call pays a capture (the served form prepares a sweep's
  // labeller when the sweep opens). The kernels are loaded first: a capture
  // must not be what loads them.
  int prepare(int max_nb) {
    if (load_label_kernels() != cudaSuccess)
      return fail(cudaGetLastError(), "loading the labeller's kernels");
    for (int c = 0; c < 2 && use_graphs; c++)
      for (int nb = 1; nb <= max_nb && nb <= kLabelMaxBatch && use_graphs; nb++)
        graph_for(nb, c, own_stream, true);
    cudaStreamSynchronize(own_stream);
    return SF_OK;
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
    {
      // Granlund & Montgomery's round-up divisor for width (as in the
      // threshold's tile counts): exact for every 32-bit numerator.
      int l = 0;
      while ((1ull << l) < width)
        l++;
      a.wdiv_m = (uint32_t)(((((unsigned long long)1 << l) - width) << 32) / width + 1);
      a.wdiv_s1 = l < 1 ? (uint32_t)l : 1u;
      a.wdiv_s2 = l > 1 ? (uint32_t)(l - 1) : 0u;
    }
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
    if (call_done) {
      if ((e = cudaEventRecord(call_done, s)) != cudaSuccess ||
          (e = cudaEventSynchronize(call_done)) != cudaSuccess)
        return fail(e, "waiting for the labeller");
    } else if ((e = cudaStreamSynchronize(s)) != cudaSuccess) {
      return fail(e, "cudaStreamSynchronize");
    }
    if (host_st->error) {
      const uint32_t err = host_st->error;
      t_last_error = (err & kErrLiveFull)
                         ? "more signal pixels held open at once than the labeller's "
                           "capacity"
                     : (err & kErrOutFull) ? "labeller outputs overflowed"
                     : (err & kErrListOverflow)
                         ? "a signal list's count exceeds its capacity (the threshold "
                           "overflowed)"
                         : "a union did not settle";
      return SF_EOVERFLOW;
    }
    const uint32_t na = host_st->n_accept, npx = host_st->n_accept_pixels;
    if ((e = spots.append(d_spots, na, s)) != cudaSuccess ||
        (e = pixels.append(d_pixels, npx, s)) != cudaSuccess) {
      if (spots.refused || pixels.refused) {
        cudaGetLastError();
        t_last_error = "the sweep's spots and pixels would grow past the device-memory budget";
        return SF_EBUSY;
      }
      return fail(e, "storing the labeller's results");
    }
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

size_t label_device_bytes(size_t height, size_t capacity, size_t min_spot_size) {
  // The pools (two of frame, index, value, parent), 22 scratch words, the
  // batch's kept pixels, the member records and tags, three variance terms
  // and an edge a slot; a spot record, a candidate record and a size-order
  // entry per possible spot.
  const size_t per =
      2 * 4 * 4 + 22 * 4 + sizeof(sf_pixel) + 4 + sizeof(sf_pixel) + 3 * 8 + 8 + 1;
  const size_t spots = capacity / std::max<size_t>(min_spot_size, 1) + 1;
  const size_t rows =
      height <= kRowTableMaxRows ? (size_t)(kLabelMaxBatch + 1) * (height + 1) * 4 : 0;
  return capacity * per + spots * (sizeof(sf_spot) + sizeof(CandSpot) + 4) + rows +
         2 * kSizeBins * 4 +
         (size_t)kGrid * kBuckets * 4 + (size_t)kScanBlocks * 4 + kLabelMaxBatch * 4 +
         2 * sizeof(LabelStatus) + 2 * sizeof(BatchArgs);
}

void label_set_growth(sf_labeller *l, LabelGrowth growth) {
  if (!l)
    return;
  l->impl.spots.growth = growth;
  l->impl.pixels.growth = growth;
}

size_t label_result_bytes(const sf_labeller *l) {
  return l ? l->impl.spots.cap * sizeof(sf_spot) + l->impl.pixels.cap * sizeof(sf_pixel) : 0;
}

int label_set_blocking_wait(sf_labeller *l) {
  if (!l)
    return SF_EBADARG;
  Labeller &L = l->impl;
  if (L.call_done)
    return SF_OK;
  const cudaError_t e =
      cudaEventCreateWithFlags(&L.call_done, cudaEventBlockingSync | cudaEventDisableTiming);
  return e == cudaSuccess ? SF_OK : fail(e, "cudaEventCreate");
}

int label_prepare(sf_labeller *l, int max_batch) {
  return l ? l->impl.prepare(max_batch) : SF_EBADARG;
}

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
