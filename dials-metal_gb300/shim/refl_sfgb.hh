// refl::write (src/spots/refl.hh:53-74, refl.cc:223-351) over libsfgb: the same
// DIALS .refl file, byte for byte, from host vectors, or straight from a
// device labeller with its shoebox column built in device memory.

#ifndef SFGB_REFL_SFGB_HH
#define SFGB_REFL_SFGB_HH

#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "dials_spots.hh"
#include "refl.hh"
#include "sf_api.h"

namespace refl_sfgb {

inline sf_refl_options options(const refl::Options &o) {
  sf_refl_options r;
  sf_default_refl_options(&r);
  r.panel = o.panel;
  r.id = o.id;
  r.identifier = o.identifier.c_str();
  r.shoeboxes = o.shoeboxes ? 1 : 0;  // mxi_find --no-shoeboxes
  return r;
}

// refl::write(path, spots, pixels, width, options).
inline void write(const std::string &path, const std::vector<dials_spots::Spot> &spots,
                  const std::vector<dials_spots::Pixel> &pixels, std::size_t width,
                  const refl::Options &o) {
  const sf_refl_options r = options(o);
  if (sf_refl_write(path.c_str(), reinterpret_cast<const sf_spot *>(spots.data()),
                    spots.size(), reinterpret_cast<const sf_pixel *>(pixels.data()),
                    pixels.size(), width, &r) != SF_OK)
    throw std::runtime_error(sf_last_error());
}

// A device labeller's run, without reading its pixels back first.
inline void write(const std::string &path, const sf_labeller *labeller,
                  const refl::Options &o) {
  const sf_refl_options r = options(o);
  if (sf_label_write_refl(labeller, path.c_str(), &r) != SF_OK)
    throw std::runtime_error(sf_last_error());
}

} // namespace refl_sfgb

#endif // SFGB_REFL_SFGB_HH
