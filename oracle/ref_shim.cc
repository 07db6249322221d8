// C entry points over the reference's own CPU code, compiled in place from
// the reference tree by oracle/build_ref.sh into oracle/_ref/libref.so.
// TEST INFRASTRUCTURE ONLY: it validates the oracle restatement and produces
// the golden fixtures under tests/golden/. It never ships and never runs on
// the GPU host (the reference tree is not there).
//
// Wrapped:
//   dext<T>()                       src/spots/dext.cc:9
//   dials_spots::Labeller           src/spots/dials_spots.hh:108-158
//   refl::write                     src/spots/refl.hh:72-74
//   synthetic::make_frame           tests/spots/synthetic_frame.hh:93-157
//   make<T>() of the fused test     tests/spots/test_dext_fused.cc:25-75

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "dext.hh"
#include "dials_spots.hh"
#include "refl.hh"
#include "signal_pixel.hh"
#include "synthetic_frame.hh"

// The fused test's frame generator lives in an anonymous namespace of a test
// program; including the program with its main renamed makes it callable here.
#define main ref_test_dext_fused_main
#include "test_dext_fused.cc"
#undef main

extern "C" {

int ref_dext_u32(const std::uint32_t *image, std::size_t h, std::size_t w,
                 SignalPixel *out, std::size_t cap, std::size_t *found) {
  std::vector<SignalPixel> signal;
  const int rc = dext<std::uint32_t>(image, signal, h, w);
  *found = signal.size();
  if (rc != 0)
    return rc;
  if (signal.size() > cap)
    return -2;
  if (!signal.empty())
    std::memcpy(out, signal.data(), signal.size() * sizeof(SignalPixel));
  return 0;
}

int ref_dext_u16(const std::uint16_t *image, std::size_t h, std::size_t w,
                 SignalPixel *out, std::size_t cap, std::size_t *found) {
  std::vector<SignalPixel> signal;
  const int rc = dext<std::uint16_t>(image, signal, h, w);
  *found = signal.size();
  if (rc != 0)
    return rc;
  if (signal.size() > cap)
    return -2;
  if (!signal.empty())
    std::memcpy(out, signal.data(), signal.size() * sizeof(SignalPixel));
  return 0;
}

// synthetic::make_frame, 16-bit pixels.
int ref_make_frame(std::size_t h, std::size_t w, std::uint64_t seed,
                   double background, int with_mask, std::uint16_t *out) {
  const synthetic::Frame f =
      synthetic::make_frame("fixture", h, w, seed, background, with_mask != 0);
  std::memcpy(out, f.pixels.data(), h * w * sizeof(std::uint16_t));
  return 0;
}

// make<T>() of test_dext_fused.cc.
int ref_fused_make_u16(std::size_t h, std::size_t w, unsigned seed, double mean,
                       std::uint16_t *out) {
  const std::vector<std::uint16_t> f = make<std::uint16_t>(h, w, seed, mean);
  std::memcpy(out, f.data(), h * w * sizeof(std::uint16_t));
  return 0;
}
int ref_fused_make_u32(std::size_t h, std::size_t w, unsigned seed, double mean,
                       std::uint32_t *out) {
  const std::vector<std::uint32_t> f = make<std::uint32_t>(h, w, seed, mean);
  std::memcpy(out, f.data(), h * w * sizeof(std::uint32_t));
  return 0;
}

struct RefLabeller {
  dials_spots::Labeller labeller;
  std::size_t width;
  std::string error;
};

void *ref_label_open(std::size_t h, std::size_t w, std::size_t min_size,
                     std::size_t max_size, double max_separation, int two_d) {
  dials_spots::Options o;
  o.min_spot_size = min_size;
  o.max_spot_size = max_size;
  o.max_separation = max_separation;
  o.two_d = two_d != 0;
  try {
    return new RefLabeller{dials_spots::Labeller(h, w, o), w, {}};
  } catch (...) {
    return nullptr;
  }
}

int ref_label_add(void *handle, std::int64_t frame, const SignalPixel *signal,
                  std::size_t n) {
  RefLabeller *l = static_cast<RefLabeller *>(handle);
  try {
    l->labeller.add(frame, std::vector<SignalPixel>(signal, signal + n));
  } catch (const std::exception &e) {
    l->error = e.what();
    return -1;
  }
  return 0;
}

void ref_label_finish(void *handle) {
  static_cast<RefLabeller *>(handle)->labeller.finish();
}

std::size_t ref_label_n_spots(void *handle) {
  return static_cast<RefLabeller *>(handle)->labeller.spots().size();
}
std::size_t ref_label_n_pixels(void *handle) {
  return static_cast<RefLabeller *>(handle)->labeller.pixels().size();
}

// Spots are copied out field by field into the oracle's or_spot layout.
struct FlatSpot {
  std::int32_t bbox[6];
  double position[3];
  double variance[3];
  double intensity;
  double intensity_variance;
  std::uint32_t n_signal;
  std::uint64_t first;
};

void ref_label_spots(void *handle, FlatSpot *out) {
  const auto &spots = static_cast<RefLabeller *>(handle)->labeller.spots();
  for (std::size_t i = 0; i < spots.size(); i++) {
    const dials_spots::Spot &s = spots[i];
    FlatSpot &f = out[i];
    std::memcpy(f.bbox, s.bbox, sizeof(f.bbox));
    std::memcpy(f.position, s.position, sizeof(f.position));
    std::memcpy(f.variance, s.variance, sizeof(f.variance));
    f.intensity = s.intensity;
    f.intensity_variance = s.intensity_variance;
    f.n_signal = s.n_signal;
    f.first = s.first;
  }
}

void ref_label_pixels(void *handle, dials_spots::Pixel *out) {
  const auto &pixels = static_cast<RefLabeller *>(handle)->labeller.pixels();
  if (!pixels.empty())
    std::memcpy(out, pixels.data(), pixels.size() * sizeof(dials_spots::Pixel));
}

void ref_label_counts(void *handle, std::uint64_t out[6]) {
  const auto &c = static_cast<RefLabeller *>(handle)->labeller.counts();
  out[0] = c.signal_pixels;
  out[1] = c.groups;
  out[2] = c.too_small;
  out[3] = c.too_large;
  out[4] = c.separated;
  out[5] = c.accepted;
}

int ref_label_write_refl_opts(void *handle, const char *path, int shoeboxes, int id,
                              const char *identifier, size_t panel) {
  RefLabeller *l = static_cast<RefLabeller *>(handle);
  refl::Options o;
  o.shoeboxes = shoeboxes != 0;
  o.id = id;
  o.identifier = identifier ? identifier : "";
  o.panel = panel;
  try {
    refl::write(path, l->labeller.spots(), l->labeller.pixels(), l->width, o);
  } catch (const std::exception &e) {
    l->error = e.what();
    return -1;
  }
  return 0;
}

int ref_label_write_refl(void *handle, const char *path, int shoeboxes) {
  RefLabeller *l = static_cast<RefLabeller *>(handle);
  refl::Options o;
  o.shoeboxes = shoeboxes != 0;
  try {
    refl::write(path, l->labeller.spots(), l->labeller.pixels(), l->width, o);
  } catch (const std::exception &e) {
    l->error = e.what();
    return -1;
  }
  return 0;
}

void ref_label_close(void *handle) { delete static_cast<RefLabeller *>(handle); }

} // extern "C"
