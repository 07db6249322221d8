// dials_spots::Labeller (src/spots/dials_spots.hh:108-125, dials_spots.cc:21-360)
// over libsfgb's device labeller. The same life cycle (construct, add frames in
// ascending order, finish, read spots / pixels / counts) and the same records,
// so mxi_find's main thread (find_spots.cc:848-891) swaps the class and keeps
// its calls; refl::write then takes spots() and pixels() unchanged.
//
// Where the reference throws std::runtime_error (an out-of-order frame, a list
// off the frame), add() throws with the library's text; a device failure or a
// full live pool throws too, since the reference has no return code there.

#ifndef SFGB_DIALS_SPOTS_SFGB_HH
#define SFGB_DIALS_SPOTS_SFGB_HH

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "dials_spots.hh"
#include "sf_api.h"

namespace dials_spots_sfgb {

static_assert(sizeof(dials_spots::Spot) == sizeof(sf_spot), "Spot layout");
static_assert(sizeof(dials_spots::Pixel) == sizeof(sf_pixel), "Pixel layout");
static_assert(sizeof(SignalPixel) == sizeof(sf_signal_pixel), "SignalPixel layout");

class Labeller {
 public:
  // live_capacity: open pixels the device holds at once (0: the library's
  // default); exceeding it fails the add that overflowed.
  Labeller(std::size_t height, std::size_t width, const dials_spots::Options &options,
           std::size_t live_capacity = 0) {
    sf_label_options lo;
    sf_default_label_options(&lo);
    lo.min_spot_size = options.min_spot_size;  // mxi_find --min-spot-size
    lo.max_spot_size = options.max_spot_size;
    lo.max_separation = options.max_separation;
    lo.two_d = options.two_d ? 1 : 0;
    l_ = sf_label_open(height, width, &lo, live_capacity);
    if (!l_)
      throw std::runtime_error(sf_last_error());
  }
  ~Labeller() { sf_label_close(l_); }
  Labeller(const Labeller &) = delete;
  Labeller &operator=(const Labeller &) = delete;

  void add(std::int64_t frame, const std::vector<SignalPixel> &signal) {
    if (sf_label_add(l_, frame, reinterpret_cast<const sf_signal_pixel *>(signal.data()),
                     signal.size()) != SF_OK)
      throw std::runtime_error(sf_last_error());
  }

  // Frames whose lists are already on the device (a plan's or a batch's
  // outputs), labelled without coming back to the host.
  void add_device(const std::int64_t *frames, std::size_t n_frames,
                  const sf_signal_pixel *d_lists, std::size_t list_stride,
                  const std::uint32_t *d_counts, void *stream) {
    if (sf_label_add_device(l_, frames, n_frames, d_lists, list_stride, d_counts, stream) !=
        SF_OK)
      throw std::runtime_error(sf_last_error());
  }

  void finish() {
    if (sf_label_finish(l_) != SF_OK)
      throw std::runtime_error(sf_last_error());
  }

  // Copies of the device-resident results (the reference returns references
  // to its own vectors).
  std::vector<dials_spots::Spot> spots() const {
    std::vector<dials_spots::Spot> s(sf_label_n_spots(l_));
    if (sf_label_spots(l_, reinterpret_cast<sf_spot *>(s.data()), s.size()) != SF_OK)
      throw std::runtime_error(sf_last_error());
    return s;
  }
  std::vector<dials_spots::Pixel> pixels() const {
    std::vector<dials_spots::Pixel> p(sf_label_n_pixels(l_));
    if (sf_label_pixels(l_, reinterpret_cast<sf_pixel *>(p.data()), p.size()) != SF_OK)
      throw std::runtime_error(sf_last_error());
    return p;
  }
  dials_spots::Counts counts() const {
    sf_counts c;
    sf_label_counts(l_, &c);
    dials_spots::Counts r;
    r.signal_pixels = c.signal_pixels;
    r.groups = c.groups;
    r.too_small = c.too_small;
    r.too_large = c.too_large;
    r.separated = c.separated;
    r.accepted = c.accepted;
    return r;
  }
  std::size_t live() const { return sf_label_live(l_); }

  // For sf_label_write_refl (refl_sfgb.hh): the file straight from the device.
  const sf_labeller *handle() const { return l_; }

 private:
  sf_labeller *l_ = nullptr;
};

} // namespace dials_spots_sfgb

#endif // SFGB_DIALS_SPOTS_SFGB_HH
