// The backend half of the reference's `namespace gpu` (src/spots/dext_gpu.hh:25-182)
// over libsfgb's C ABI. It takes the place of src/spots/dext_cuda.cu in a
// SPOTFINDER_CUDA build (cmake/spots.cmake:406-420); src/spots/dext_gpu.cc, the
// policy half (windows, profiling flag, announcements), is linked unchanged.
//
// Build: compile with the reference's src/spots on the include path and
// libsfgb's include/ beside it, and link -lsfgb (and -lcudart).
//
// find<T> (dext_gpu.hh:171-180, dext_cuda.cu:711-869): the device writes the
// ascending signal list of at most capacity = one record per 16 bytes of
// frame (the reference's device bound, dext_cuda.cu:741) into this thread's
// page-locked staging buffer, and only the records found are copied into
// signal_out, as dext_cuda.cu:841-846 resizes to the count it reads back.
// Neither the staging buffer nor signal_out is filled to capacity, so a 16M
// 32-bit frame costs a copy of its ~2 MB of records, not a 72 MB fill.

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "dext_gpu.hh"
#include "dext_gpu_internal.hh"
#include "sf_api.h"

namespace gpu {

namespace {

static_assert(sizeof(SignalPixel) == sizeof(sf_signal_pixel), "SignalPixel layout");

// One staging buffer per calling thread, page-locked so that the list's copy
// back is asynchronous, grown to the largest capacity asked for and kept for
// the thread's life (mxi_find's workers call find() once a frame).
class Staging {
 public:
  ~Staging() { sf_host_free(data_); }
  sf_signal_pixel *reserve(std::size_t records) {
    if (records > capacity_) {
      sf_host_free(data_);
      data_ = static_cast<sf_signal_pixel *>(sf_host_alloc(records * sizeof(sf_signal_pixel)));
      capacity_ = data_ ? records : 0;
    }
    return data_;
  }

 private:
  sf_signal_pixel *data_ = nullptr;
  std::size_t capacity_ = 0;
};

Staging &staging() {
  static thread_local Staging s;
  return s;
}

} // namespace

const char *backend() { return sf_backend(); }
bool available() { return sf_available() != 0; }
std::string unavailable_reason() { return sf_unavailable_reason(); }
std::size_t memory_free() { return sf_memory_free(); }
void *host_alloc(std::size_t bytes) { return sf_host_alloc(bytes); }
void host_free(void *pointer) { sf_host_free(pointer); }

namespace internal {
// The three stages run as one launch sequence here, so there is no window to
// choose; dext_gpu.cc still reads and announces the setting.
Window default_stage0_window() { return Window::Tile; }
Window default_stage2_window() { return Window::Tile; }
} // namespace internal

template <typename T>
int find(const T *image_in, std::vector<SignalPixel> &signal_out, std::size_t height,
         std::size_t width) {
  signal_out.clear();
  const std::size_t capacity = height * width * sizeof(T) / 16;
  sf_profile_stages(profile_stages() ? 1 : 0);
  sf_signal_pixel *out = nullptr;
  if (image_in && capacity) {
    out = staging().reserve(capacity);
    if (!out)
      throw std::runtime_error("CUDA: page-locked staging of " +
                               std::to_string(capacity * sizeof(sf_signal_pixel)) +
                               " bytes failed");
  }
  std::size_t found = 0;
  int rc;
  if constexpr (sizeof(T) == 4)
    rc = sf_find_u32(reinterpret_cast<const std::uint32_t *>(image_in), height, width, out,
                     capacity, &found);
  else
    rc = sf_find_u16(reinterpret_cast<const std::uint16_t *>(image_in), height, width, out,
                     capacity, &found);
  // The reference throws on a device failure (dext_cuda.cu:46-51) and returns
  // -1 / -2 for a bad argument / a list beyond its bound.
  if (rc != SF_OK && rc != SF_EBADARG && rc != SF_EOVERFLOW)
    throw std::runtime_error(std::string("CUDA: ") + sf_last_error());
  if (rc == SF_OK && found) {
    signal_out.resize(found);
    std::memcpy(static_cast<void *>(signal_out.data()), out, found * sizeof(SignalPixel));
  }
  if (profile_stages()) {
    sf_stage_times t;
    sf_last_stage_times(&t);
    StageTimes s;
    s.upload = t.upload;
    s.stage0 = t.stage0;
    s.stage1 = t.stage1;
    s.stage2 = t.stage2;
    s.fused = t.fused;
    s.copy = t.copy;
    s.sort = t.sort;
    internal::set_stage_times(s);
  }
  return rc;
}

template int find<std::uint16_t>(const std::uint16_t *, std::vector<SignalPixel> &, std::size_t,
                                 std::size_t);
template int find<std::uint32_t>(const std::uint32_t *, std::vector<SignalPixel> &, std::size_t,
                                 std::size_t);

} // namespace gpu
