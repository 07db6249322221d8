// The DIALS reflection table (.refl) of a spot-finding run, written as the
// reference's refl::write (src/spots/refl.hh:72-74, refl.cc:223-351) writes
// it, byte for byte.
//
// A .refl file is one msgpack document:
//
//   [ "dials::af::reflection_table", 2,
//     { "identifiers": { id: identifier } or {},
//       "nrows": N,
//       "data": { column name: [ type name, [ N, bin(raw column) ] ], ... } } ]
//
// with the columns of dials.find_spots in name order: bbox (int6), flags
// (std::size_t, Strong), id (int), intensity.sum.value and .variance
// (double), n_signal (int), panel (std::size_t), shoebox (Shoebox<>, when
// asked for), xyzobs.px.value and .variance (vec3<double>). Every payload is a
// little-endian memory image. Integers, strings, arrays, maps and binary
// lengths take the shortest msgpack form that holds them, as the reference's
// writer chooses them.
//
// The shoebox column is the only large one: per spot the panel (uint32), the
// bbox (6 x int32), a version byte (2), then over the box (z slowest, x
// fastest) float data, a byte mask and a float background. The spot finder
// fills only its signal pixels (data = the value, mask = valid | foreground)
// and leaves the rest, and the whole background, at zero.
//
// Two entry points share one encoder: sf_refl_write takes host spot and pixel
// arrays and needs no GPU; sf_label_write_refl takes a device labeller, builds
// the shoebox column in device memory from the labeller's device-resident
// pixels (one warp a spot) and copies it out in one piece.

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "sf_api.h"
#include "sf_label.cuh"

namespace sf {

extern thread_local std::string t_last_error;
int fail(cudaError_t e, const char *what);

namespace {

constexpr uint8_t kMaskValidForeground = 1u | 4u;  // DIALS mask codes Valid, Foreground
constexpr uint64_t kFlagStrong = 1ull << 5;          // dials::af::Flags::Strong
constexpr size_t kShoeboxHead = 4 + 6 * 4 + 1;       // panel, bbox, version

static_assert(sizeof(float) == 4 && sizeof(double) == 8, "IEEE float and double");

uint64_t box_elements(const sf_spot &s) {
  return (uint64_t)(s.bbox[1] - s.bbox[0]) * (uint64_t)(s.bbox[3] - s.bbox[2]) *
         (uint64_t)(s.bbox[5] - s.bbox[4]);
}

uint64_t shoebox_bytes(const sf_spot &s) { return kShoeboxHead + box_elements(s) * 9; }

// Buffered file output; false once anything failed.
struct Sink {
  FILE *f = nullptr;
  std::vector<uint8_t> buf;
  bool ok = true;
  explicit Sink(const char *path) : f(fopen(path, "wb")) {
    ok = f != nullptr;
    buf.reserve(1 << 20);
  }
  ~Sink() {
    if (f)
      fclose(f);
  }
  void put(const void *p, size_t n) {
    const uint8_t *b = static_cast<const uint8_t *>(p);
    if (n >= (1u << 20)) {
      drain();
      if (ok && fwrite(b, 1, n, f) != n)
        ok = false;
      return;
    }
    buf.insert(buf.end(), b, b + n);
    if (buf.size() >= (1u << 20))
      drain();
  }
  void u8(uint8_t v) { put(&v, 1); }
  void drain() {
    if (ok && !buf.empty() && fwrite(buf.data(), 1, buf.size(), f) != buf.size())
      ok = false;
    buf.clear();
  }
  bool finish() {
    drain();
    if (f && fclose(f) != 0)
      ok = false;
    f = nullptr;
    return ok;
  }
};

// msgpack headers: a marker byte, then a big-endian length or value.
void big_endian(Sink &o, uint64_t v, int bytes) {
  uint8_t b[8];
  for (int i = 0; i < bytes; i++)
    b[i] = (uint8_t)(v >> (8 * (bytes - 1 - i)));
  o.put(b, (size_t)bytes);
}

void mp_uint(Sink &o, uint64_t v) {
  if (v < 0x80) {
    o.u8((uint8_t)v);
    return;
  }
  const int bytes = v <= 0xFF ? 1 : v <= 0xFFFF ? 2 : v <= 0xFFFFFFFFull ? 4 : 8;
  o.u8(bytes == 1 ? 0xCC : bytes == 2 ? 0xCD : bytes == 4 ? 0xCE : 0xCF);
  big_endian(o, v, bytes);
}

void mp_str(Sink &o, const char *s, size_t n) {
  if (n < 32) {
    o.u8((uint8_t)(0xA0 | n));
  } else {
    const int bytes = n <= 0xFF ? 1 : n <= 0xFFFF ? 2 : 4;
    o.u8(bytes == 1 ? 0xD9 : bytes == 2 ? 0xDA : 0xDB);
    big_endian(o, n, bytes);
  }
  o.put(s, n);
}

void mp_str(Sink &o, const char *s) { mp_str(o, s, strlen(s)); }

// fix (below 16), 16- or 32-bit count: base 0x90 (array) or 0x80 (map).
void mp_count(Sink &o, size_t n, uint8_t fix, uint8_t c16, uint8_t c32) {
  if (n < 16) {
    o.u8((uint8_t)(fix | n));
  } else if (n <= 0xFFFF) {
    o.u8(c16);
    big_endian(o, n, 2);
  } else {
    o.u8(c32);
    big_endian(o, n, 4);
  }
}
void mp_array(Sink &o, size_t n) { mp_count(o, n, 0x90, 0xDC, 0xDD); }
void mp_map(Sink &o, size_t n) { mp_count(o, n, 0x80, 0xDE, 0xDF); }

void mp_bin(Sink &o, uint64_t n) {
  const int bytes = n <= 0xFF ? 1 : n <= 0xFFFF ? 2 : 4;
  o.u8(bytes == 1 ? 0xC4 : bytes == 2 ? 0xC5 : 0xC6);
  big_endian(o, n, bytes);
}

// name: [ type, [ rows, bin(bytes) ] ]; the payload follows.
void column(Sink &o, const char *name, const char *type, size_t rows, uint64_t bytes) {
  mp_str(o, name);
  mp_array(o, 2);
  mp_str(o, type);
  mp_array(o, 2);
  mp_uint(o, rows);
  mp_bin(o, bytes);
}

template <typename T> void raw(Sink &o, T v) { o.put(&v, sizeof(T)); }

// The host shoebox of one spot, appended to `out`.
void host_shoebox(const sf_spot &s, const sf_pixel *pixels, size_t width, uint32_t panel,
                  std::vector<uint8_t> *out) {
  const size_t xs = (size_t)(s.bbox[1] - s.bbox[0]), ys = (size_t)(s.bbox[3] - s.bbox[2]);
  const size_t n = (size_t)box_elements(s);
  const size_t at0 = out->size();
  out->resize(at0 + kShoeboxHead + 9 * n, 0);
  uint8_t *b = out->data() + at0;
  memcpy(b, &panel, 4);
  memcpy(b + 4, s.bbox, 24);
  b[28] = 2;  // shoebox version 2: a byte mask
  uint8_t *data = b + kShoeboxHead, *mask = data + 4 * n;
  for (uint32_t k = 0; k < s.n_signal; k++) {
    const sf_pixel &p = pixels[s.first + k];
    const size_t x = (size_t)(p.index % width) - (size_t)s.bbox[0];
    const size_t y = (size_t)(p.index / width) - (size_t)s.bbox[2];
    const size_t z = (size_t)((int64_t)p.frame - s.bbox[4]);
    const size_t at = (z * ys + y) * xs + x;
    const float v = (float)p.value;
    memcpy(data + 4 * at, &v, 4);
    mask[at] = kMaskValidForeground;
  }
}

// The whole document; `shoebox` supplies the shoebox column's bytes in spot
// order (total `sb_bytes`) when options->shoeboxes is set.
template <class Shoebox>
int encode(const char *path, const sf_spot *spots, size_t rows, const sf_refl_options &op,
           uint64_t sb_bytes, Shoebox shoebox) {
  if (op.shoeboxes && sb_bytes > 0xFFFFFFFFull) {
    t_last_error = "the shoebox column would be over 4 GB, more than msgpack's binary type "
                   "can hold; write without shoeboxes";
    return SF_EUNSUPPORTED;
  }
  Sink o(path);
  if (!o.ok) {
    t_last_error = std::string("cannot write ") + path;
    return SF_EBADARG;
  }
  mp_array(o, 3);
  mp_str(o, "dials::af::reflection_table");
  mp_uint(o, 2);
  mp_map(o, 3);
  mp_str(o, "identifiers");
  const char *ident = op.identifier ? op.identifier : "";
  if (ident[0]) {
    mp_map(o, 1);
    mp_uint(o, (uint64_t)(int64_t)op.id);  // as the reference casts it
    mp_str(o, ident);
  } else {
    mp_map(o, 0);
  }
  mp_str(o, "nrows");
  mp_uint(o, rows);
  mp_str(o, "data");
  mp_map(o, op.shoeboxes ? 10 : 9);
  column(o, "bbox", "int6", rows, (uint64_t)rows * 24);
  for (size_t i = 0; i < rows; i++)
    o.put(spots[i].bbox, 24);
  column(o, "flags", "std::size_t", rows, (uint64_t)rows * 8);
  for (size_t i = 0; i < rows; i++)
    raw<uint64_t>(o, kFlagStrong);
  column(o, "id", "int", rows, (uint64_t)rows * 4);
  for (size_t i = 0; i < rows; i++)
    raw<int32_t>(o, op.id);
  column(o, "intensity.sum.value", "double", rows, (uint64_t)rows * 8);
  for (size_t i = 0; i < rows; i++)
    raw<double>(o, spots[i].intensity);
  column(o, "intensity.sum.variance", "double", rows, (uint64_t)rows * 8);
  for (size_t i = 0; i < rows; i++)
    raw<double>(o, spots[i].intensity_variance);
  column(o, "n_signal", "int", rows, (uint64_t)rows * 4);
  for (size_t i = 0; i < rows; i++)
    raw<int32_t>(o, (int32_t)spots[i].n_signal);
  column(o, "panel", "std::size_t", rows, (uint64_t)rows * 8);
  for (size_t i = 0; i < rows; i++)
    raw<uint64_t>(o, (uint64_t)op.panel);
  if (op.shoeboxes) {
    column(o, "shoebox", "Shoebox<>", rows, sb_bytes);
    const int rc = shoebox(o);
    if (rc != SF_OK)
      return rc;
  }
  column(o, "xyzobs.px.value", "vec3<double>", rows, (uint64_t)rows * 24);
  for (size_t i = 0; i < rows; i++)
    o.put(spots[i].position, 24);
  column(o, "xyzobs.px.variance", "vec3<double>", rows, (uint64_t)rows * 24);
  for (size_t i = 0; i < rows; i++)
    o.put(spots[i].variance, 24);
  if (!o.finish()) {
    t_last_error = std::string("cannot finish writing ") + path;
    return SF_EBADARG;
  }
  return SF_OK;
}

bool spots_fit(const sf_spot *spots, size_t rows, size_t n_pixels) {
  for (size_t i = 0; i < rows; i++) {
    const sf_spot &s = spots[i];
    if (s.bbox[1] < s.bbox[0] || s.bbox[3] < s.bbox[2] || s.bbox[5] < s.bbox[4] ||
        s.first > n_pixels || s.n_signal > n_pixels - s.first)
      return false;
  }
  return true;
}

// One warp a spot: lane 0 writes the head, the lanes scatter the spot's
// pixels into the zeroed box (data as float, mask valid | foreground).
__global__ void __launch_bounds__(256)
k_shoeboxes(const sf_spot *__restrict__ spots, const unsigned long long *__restrict__ offset,
            size_t rows, const sf_pixel *__restrict__ pixels, uint32_t width, uint32_t panel,
            uint8_t *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  for (size_t i = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < rows;
       i += ((size_t)gridDim.x * blockDim.x) >> 5) {
    const sf_spot s = spots[i];
    uint8_t *b = out + offset[i];
    const uint32_t xs = (uint32_t)(s.bbox[1] - s.bbox[0]),
                   ys = (uint32_t)(s.bbox[3] - s.bbox[2]);
    const size_t n = (size_t)xs * ys * (uint32_t)(s.bbox[5] - s.bbox[4]);
    if (lane == 0) {
      memcpy(b, &panel, 4);
      memcpy(b + 4, s.bbox, 24);
      b[28] = 2;
    }
    uint8_t *data = b + kShoeboxHead, *mask = data + 4 * n;
    for (uint32_t k = lane; k < s.n_signal; k += 32) {
      const sf_pixel p = pixels[s.first + k];
      const uint32_t x = p.index % width - (uint32_t)s.bbox[0];
      const uint32_t y = p.index / width - (uint32_t)s.bbox[2];
      const uint32_t z = (uint32_t)(p.frame - s.bbox[4]);
      const size_t at = ((size_t)z * ys + y) * xs + x;
      const float v = __uint2float_rn(p.value);  // the host's static_cast<float>
      uint32_t bits;
      memcpy(&bits, &v, 4);
      uint8_t *d = data + 4 * at;  // not 4-byte aligned in the column
      d[0] = (uint8_t)bits;
      d[1] = (uint8_t)(bits >> 8);
      d[2] = (uint8_t)(bits >> 16);
      d[3] = (uint8_t)(bits >> 24);
      mask[at] = kMaskValidForeground;
    }
  }
}

struct DeviceBuffers {
  void *p[4] = {nullptr, nullptr, nullptr, nullptr};
  ~DeviceBuffers() {
    for (void *q : p)
      cudaFree(q);
  }
};

} // namespace
} // namespace sf

extern "C" {

void sf_default_refl_options(sf_refl_options *o) {
  if (!o)
    return;
  o->panel = 0;
  o->id = 0;
  o->identifier = nullptr;
  o->shoeboxes = 1;
}

int sf_refl_write(const char *path, const sf_spot *spots, size_t n_spots,
                  const sf_pixel *pixels, size_t n_pixels, size_t width,
                  const sf_refl_options *options) {
  using namespace sf;
  sf_refl_options op;
  sf_default_refl_options(&op);
  if (options)
    op = *options;
  if (!path || width == 0 || width > 0xFFFFFFFFull || (n_spots && !spots) ||
      (n_pixels && !pixels) || !spots_fit(spots, n_spots, n_pixels)) {
    t_last_error = "sf_refl_write: no path, a zero width, or spots whose pixels or boxes are "
                   "not in the arrays given";
    return SF_EBADARG;
  }
  uint64_t sb = 0;
  for (size_t i = 0; i < n_spots; i++)
    sb += shoebox_bytes(spots[i]);
  return encode(path, spots, n_spots, op, sb, [&](Sink &o) {
    std::vector<uint8_t> box;
    for (size_t i = 0; i < n_spots; i++) {
      box.clear();
      host_shoebox(spots[i], pixels, width, (uint32_t)op.panel, &box);
      o.put(box.data(), box.size());
    }
    return SF_OK;
  });
}

int sf_label_write_refl(const sf_labeller *labeller, const char *path,
                        const sf_refl_options *options) {
  using namespace sf;
  sf_refl_options op;
  sf_default_refl_options(&op);
  if (options)
    op = *options;
  if (!labeller || !path) {
    t_last_error = "sf_label_write_refl: no labeller or no path";
    return SF_EBADARG;
  }
  const size_t rows = sf_label_n_spots(labeller), npix = sf_label_n_pixels(labeller);
  const size_t width = label_width(labeller);
  std::vector<sf_spot> spots(rows);
  int rc = sf_label_spots(labeller, spots.data(), rows);
  if (rc != SF_OK)
    return rc;
  if (!spots_fit(spots.data(), rows, npix)) {
    t_last_error = "sf_label_write_refl: the labeller's spots do not match its pixels";
    return SF_EBADARG;
  }
  std::vector<unsigned long long> offset(rows);
  uint64_t sb = 0;
  for (size_t i = 0; i < rows; i++) {
    offset[i] = sb;
    sb += shoebox_bytes(spots[i]);
  }
  return encode(path, spots.data(), rows, op, sb, [&](Sink &o) {
    if (rows == 0)
      return SF_OK;
    // The column in device memory: zeroed, then each spot's head and pixels.
    DeviceBuffers d;
    cudaStream_t s = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&d.p[0], npix * sizeof(sf_pixel) + 1)) != cudaSuccess ||
        (e = cudaMalloc(&d.p[1], rows * sizeof(sf_spot))) != cudaSuccess ||
        (e = cudaMalloc(&d.p[2], rows * sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaMalloc(&d.p[3], sb)) != cudaSuccess)
      return fail(e, "allocating the shoebox column");
    int r = label_gather_pixels(labeller, static_cast<sf_pixel *>(d.p[0]), &s);
    if (r != SF_OK)
      return r;
    std::vector<uint8_t> host(sb);
    const unsigned blocks = (unsigned)std::min<size_t>((rows + 7) / 8, 4096);
    if ((e = cudaMemcpyAsync(d.p[1], spots.data(), rows * sizeof(sf_spot),
                             cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d.p[2], offset.data(), rows * sizeof(unsigned long long),
                             cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(d.p[3], 0, sb, s)) != cudaSuccess)
      return fail(e, "preparing the shoebox column");
    k_shoeboxes<<<blocks, 256, 0, s>>>(static_cast<const sf_spot *>(d.p[1]),
                                       static_cast<const unsigned long long *>(d.p[2]), rows,
                                       static_cast<const sf_pixel *>(d.p[0]), (uint32_t)width,
                                       (uint32_t)op.panel, static_cast<uint8_t *>(d.p[3]));
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(host.data(), d.p[3], sb, cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      return fail(e, "building the shoebox column");
    o.put(host.data(), host.size());
    return SF_OK;
  });
}

} // extern "C"
