// The served form (include/sf_api.h, sf_server_*): a request loop for frames
// that arrive from several detector streams at once.
//
// Every open sweep keeps its state on the device: a ring of frame slots and
// its 3-D labeller (the open components and their pixels, dials_spots.cc).
// Sweeps are admitted against a device-memory budget. One worker thread runs
// the loop:
//   1. submitted host frames go to free slots of their sweep, copied on a
//      copy stream while the GPU computes;
//   2. frames already on the device form a batch (continuous batching: what
//      is ready now, across sweeps of one frame shape and parameter set, up
//      to max_batch) and one threshold launch sequence handles it on the
//      compute stream, into one of two output sets;
//   3. meanwhile the previous batch is labelled, each sweep's frames in
//      frame order, on a label stream; when that finishes its frames are done
//      (latency: submit to labelled) and their slots are free again.
// A frame's result does not depend on what shares its batch: every frame is
// thresholded alone within a batch and each sweep's labeller sees only its
// own frames, in order.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sf_api.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct SrvFrame {
  int64_t sweep = 0, number = 0;
  const uint32_t *host = nullptr;
  double t_submit = 0.0;
  int slot = -1;
  cudaEvent_t up = nullptr;  // upload done
};

// Frames of one shape and parameter set share launches and outputs.
struct SrvGroup {
  size_t h = 0, w = 0, capacity = 0;
  sf_threshold_params params{};
  void *ws = nullptr;
  size_t ws_bytes = 0;
  sf_signal_pixel *out[2] = {nullptr, nullptr};
  uint32_t *counts[2] = {nullptr, nullptr}, *bits[2] = {nullptr, nullptr};
  uint32_t *host_counts = nullptr;  // pinned, max_batch
  int next = 0, users = 0;
  size_t bytes = 0;
  ~SrvGroup() {
    cudaFree(ws);
    for (int i = 0; i < 2; i++) {
      cudaFree(out[i]);
      cudaFree(counts[i]);
      cudaFree(bits[i]);
    }
    if (host_counts)
      cudaFreeHost(host_counts);
  }
};

struct SrvSweep {
  int64_t id = 0;
  SrvGroup *group = nullptr;
  sf_labeller *lab = nullptr;
  size_t bytes = 0;
  std::vector<uint32_t *> slots;
  std::vector<int> free_slots;
  std::deque<SrvFrame> pending;   // submitted, waiting for a slot
  std::deque<SrvFrame> uploaded;  // on the device, waiting for a batch
  size_t in_flight = 0;           // submitted and not yet done
  int64_t last_number = LLONG_MIN;
  bool finishing = false, finished = false;
  int status = 0;
  ~SrvSweep() {
    if (lab)
      sf_label_close(lab);
    for (uint32_t *p : slots)
      cudaFree(p);
  }
};

struct SrvBatch {
  SrvGroup *g = nullptr;
  int buf = 0;
  std::vector<SrvFrame> frames;  // grouped by sweep, in frame order
  cudaEvent_t done = nullptr;
};

} // namespace

struct sf_server {
  sf_server_options opt{};
  int device = 0;
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::map<int64_t, std::unique_ptr<SrvSweep>> sweeps;
  std::vector<std::unique_ptr<SrvGroup>> groups;
  std::deque<sf_frame_done> done;
  std::vector<cudaEvent_t> event_pool;
  std::thread worker;
  bool stop = false;
  int64_t next_id = 1;
  size_t used = 0;
  cudaStream_t copy_s = nullptr, comp_s = nullptr, label_s = nullptr;
  std::string error;

  cudaEvent_t get_event() {
    if (!event_pool.empty()) {
      cudaEvent_t e = event_pool.back();
      event_pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return e;
  }
  void put_event(cudaEvent_t e) {
    if (e)
      event_pool.push_back(e);
  }

  bool work_ready() {
    for (auto &kv : sweeps) {
      SrvSweep &s = *kv.second;
      if ((!s.pending.empty() && !s.free_slots.empty()) || !s.uploaded.empty())
        return true;
      if (s.finishing && !s.finished && s.in_flight == 0)
        return true;
    }
    return false;
  }

  void run();
  void label_batch(SrvBatch &b);
};

namespace {

size_t labeller_capacity(size_t h, size_t w) {
  return std::min<size_t>((size_t)1 << 22, std::max<size_t>(h * w / 2, 1024));
}

// Device bytes of a labeller of the given capacity (its pools, scratch and
// outputs, as sf_label_open allocates them), with a margin.
size_t labeller_bytes(size_t capacity, size_t min_spot_size) {
  const size_t per = 2 * 4 * 4 + 22 * 4 + 12;
  const size_t spots = capacity / std::max<size_t>(min_spot_size, 1) + 1;
  return capacity * per + spots * sizeof(sf_spot) + ((size_t)16 << 20);
}

size_t group_bytes(size_t h, size_t w, size_t capacity, size_t max_batch) {
  const size_t words = (w + 31) / 32 * h;
  return sf_batch_workspace_bytes(max_batch, h, w, capacity) +
         2 * max_batch * (capacity * sizeof(sf_signal_pixel) + words * 4 + 4);
}

bool same_params(const sf_threshold_params &a, const sf_threshold_params &b) {
  return a.algorithm == b.algorithm && a.kernel_x == b.kernel_x && a.kernel_y == b.kernel_y &&
         a.gain == b.gain && a.sigma_b == b.sigma_b && a.sigma_s == b.sigma_s &&
         a.min_local == b.min_local && a.global_threshold == b.global_threshold;
}

} // namespace

void sf_server::label_batch(SrvBatch &b) {
  // The batch's threshold is done (the label stream waits for it); each
  // sweep's run of frames goes to its labeller in order.
  cudaStreamWaitEvent(label_s, b.done, 0);
  SrvGroup &g = *b.g;
  const size_t n = b.frames.size();
  cudaMemcpyAsync(g.host_counts, g.counts[b.buf], n * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                  label_s);
  std::vector<int> status(n, 0);
  size_t j = 0;
  while (j < n) {
    size_t k = j;
    while (k < n && b.frames[k].sweep == b.frames[j].sweep)
      k++;
    SrvSweep *s = nullptr;
    {
      std::lock_guard<std::mutex> lock(m);
      auto it = sweeps.find(b.frames[j].sweep);
      s = it == sweeps.end() ? nullptr : it->second.get();
    }
    int rc = SF_EBADARG;
    if (s && s->status == 0) {
      std::vector<int64_t> numbers;
      for (size_t i = j; i < k; i++)
        numbers.push_back(b.frames[i].number);
      rc = sf_label_add_device(s->lab, numbers.data(), numbers.size(),
                               g.out[b.buf] + j * g.capacity, g.capacity, g.counts[b.buf] + j,
                               label_s);
      if (rc != SF_OK)
        s->status = rc;
    } else if (s) {
      rc = s->status;
    }
    for (size_t i = j; i < k; i++)
      status[i] = rc;
    j = k;
  }
  cudaStreamSynchronize(label_s);
  const double t = now_s();
  std::lock_guard<std::mutex> lock(m);
  for (size_t i = 0; i < n; i++) {
    SrvFrame &f = b.frames[i];
    sf_frame_done d;
    d.sweep = f.sweep;
    d.frame = f.number;
    d.n_signal = g.host_counts[i];
    d.latency_ms = (t - f.t_submit) * 1e3;
    d.status = status[i];
    done.push_back(d);
    auto it = sweeps.find(f.sweep);
    if (it != sweeps.end()) {
      it->second->free_slots.push_back(f.slot);
      it->second->in_flight--;
    }
    put_event(f.up);
  }
  put_event(b.done);
  cv_done.notify_all();
  cv_work.notify_all();
}

void sf_server::run() {
  cudaSetDevice(device);
  std::unique_ptr<SrvBatch> prev;
  while (true) {
    std::unique_ptr<SrvBatch> cur;
    std::vector<SrvSweep *> to_finish;
    {
      std::unique_lock<std::mutex> lock(m);
      cv_work.wait(lock, [&] { return stop || work_ready() || prev; });
      if (stop && !work_ready() && !prev)
        break;
      // 1. Uploads into free slots, oldest submissions first.
      for (auto &kv : sweeps) {
        SrvSweep &s = *kv.second;
        while (!s.pending.empty() && !s.free_slots.empty()) {
          SrvFrame f = s.pending.front();
          s.pending.pop_front();
          f.slot = s.free_slots.back();
          s.free_slots.pop_back();
          f.up = get_event();
          const size_t bytes = s.group->h * s.group->w * sizeof(uint32_t);
          cudaError_t e = cudaMemcpyAsync(s.slots[f.slot], f.host, bytes,
                                          cudaMemcpyHostToDevice, copy_s);
          if (e == cudaSuccess)
            e = cudaEventRecord(f.up, copy_s);
          if (e != cudaSuccess && s.status == 0)
            s.status = SF_ECUDA;
          s.uploaded.push_back(f);
        }
      }
      // 2. A batch: the shape group of the oldest frame on the device, every
      // ready frame of its sweeps up to max_batch, grouped by sweep.
      SrvSweep *first = nullptr;
      for (auto &kv : sweeps) {
        SrvSweep &s = *kv.second;
        if (!s.uploaded.empty() &&
            (!first || s.uploaded.front().t_submit < first->uploaded.front().t_submit))
          first = &s;
      }
      if (first) {
        cur.reset(new SrvBatch);
        cur->g = first->group;
        for (auto &kv : sweeps) {
          SrvSweep &s = *kv.second;
          if (s.group != cur->g)
            continue;
          while (!s.uploaded.empty() && cur->frames.size() < opt.max_batch) {
            cur->frames.push_back(s.uploaded.front());
            s.uploaded.pop_front();
          }
        }
        cur->buf = cur->g->next;
        cur->g->next ^= 1;
        cur->done = get_event();
      }
      for (auto &kv : sweeps) {
        SrvSweep &s = *kv.second;
        if (s.finishing && !s.finished && s.in_flight == 0)
          to_finish.push_back(&s);
      }
    }
    if (cur) {
      SrvGroup &g = *cur->g;
      std::vector<const uint32_t *> images;
      for (SrvFrame &f : cur->frames) {
        cudaStreamWaitEvent(comp_s, f.up, 0);
        std::lock_guard<std::mutex> lock(m);
        images.push_back(sweeps[f.sweep]->slots[f.slot]);
      }
      const int rc = sf_threshold_u32_batch_device(
          images.data(), images.size(), g.h, g.w, &g.params, g.out[cur->buf], g.capacity,
          g.bits[cur->buf], g.counts[cur->buf], nullptr, g.ws, g.ws_bytes, comp_s);
      cudaEventRecord(cur->done, comp_s);
      if (rc != SF_OK) {
        std::lock_guard<std::mutex> lock(m);
        for (SrvFrame &f : cur->frames)
          if (sweeps[f.sweep]->status == 0)
            sweeps[f.sweep]->status = rc;
      }
    }
    // 3. The previous batch is labelled while this one is thresholded.
    if (prev)
      label_batch(*prev);
    prev = std::move(cur);
    for (SrvSweep *s : to_finish) {
      const int rc = s->status == 0 ? sf_label_finish(s->lab) : s->status;
      std::lock_guard<std::mutex> lock(m);
      if (rc != SF_OK && s->status == 0)
        s->status = rc;
      s->finished = true;
      cv_done.notify_all();
    }
  }
}

extern "C" {

void sf_default_server_options(sf_server_options *o) {
  if (!o)
    return;
  o->hbm_budget = 0;
  o->max_batch = 16;
  o->ring = 32;
  o->capacity_divisor = 16;
}

sf_server *sf_server_open(const sf_server_options *options) {
  sf_server_options o;
  if (options)
    o = *options;
  else
    sf_default_server_options(&o);
  if (o.max_batch == 0 || o.max_batch > SF_MAX_BATCH || o.ring < o.max_batch ||
      o.capacity_divisor == 0)
    return nullptr;
  sf_server *sv = new sf_server();
  sv->opt = o;
  cudaGetDevice(&sv->device);
  if (sv->opt.hbm_budget == 0) {
    size_t fb = 0, tb = 0;
    cudaMemGetInfo(&fb, &tb);
    sv->opt.hbm_budget = fb / 10 * 8;
  }
  if (cudaStreamCreateWithFlags(&sv->copy_s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&sv->comp_s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&sv->label_s, cudaStreamNonBlocking) != cudaSuccess) {
    delete sv;
    return nullptr;
  }
  sv->worker = std::thread([sv] { sv->run(); });
  return sv;
}

void sf_server_close(sf_server *sv) {
  if (!sv)
    return;
  {
    std::lock_guard<std::mutex> lock(sv->m);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  if (sv->worker.joinable())
    sv->worker.join();
  cudaDeviceSynchronize();
  sv->sweeps.clear();
  sv->groups.clear();
  for (cudaEvent_t e : sv->event_pool)
    cudaEventDestroy(e);
  cudaStreamDestroy(sv->copy_s);
  cudaStreamDestroy(sv->comp_s);
  cudaStreamDestroy(sv->label_s);
  delete sv;
}

size_t sf_server_sweep_bytes(const sf_server *sv, size_t height, size_t width,
                             const sf_label_options *label) {
  if (!sv || height == 0 || width == 0)
    return 0;
  const size_t min_size = label ? label->min_spot_size : 3;
  return sv->opt.ring * height * width * sizeof(uint32_t) +
         labeller_bytes(labeller_capacity(height, width), min_size);
}

int sf_server_open_sweep(sf_server *sv, size_t height, size_t width,
                         const sf_threshold_params *params, const sf_label_options *label,
                         int64_t *sweep) {
  if (!sv || !sweep || height == 0 || width == 0 || height > 0x7fffffffu / width)
    return SF_EBADARG;
  sf_threshold_params p;
  if (params)
    p = *params;
  else
    sf_default_params(&p);
  const size_t capacity = std::max<size_t>(1, height * width / sv->opt.capacity_divisor);
  std::unique_lock<std::mutex> lock(sv->m);
  SrvGroup *g = nullptr;
  for (auto &gr : sv->groups)
    if (gr->h == height && gr->w == width && same_params(gr->params, p))
      g = gr.get();
  size_t need = sf_server_sweep_bytes(sv, height, width, label);
  const size_t gb = g ? 0 : group_bytes(height, width, capacity, sv->opt.max_batch);
  if (sv->used + need + gb > sv->opt.hbm_budget)
    return SF_EBUSY;
  lock.unlock();
  std::unique_ptr<SrvGroup> fresh;
  cudaError_t e = cudaSuccess;
  if (!g) {
    fresh.reset(new SrvGroup);
    SrvGroup &G = *fresh;
    G.h = height;
    G.w = width;
    G.params = p;
    G.capacity = capacity;
    G.bytes = gb;
    G.ws_bytes = sf_batch_workspace_bytes(sv->opt.max_batch, height, width, capacity);
    const size_t words = (width + 31) / 32 * height;
    if ((e = cudaMalloc(&G.ws, G.ws_bytes)) == cudaSuccess)
      for (int i = 0; i < 2 && e == cudaSuccess; i++) {
        e = cudaMalloc(&G.out[i], sv->opt.max_batch * capacity * sizeof(sf_signal_pixel));
        if (e == cudaSuccess)
          e = cudaMalloc(&G.counts[i], sv->opt.max_batch * sizeof(uint32_t));
        if (e == cudaSuccess)
          e = cudaMalloc(&G.bits[i], sv->opt.max_batch * words * sizeof(uint32_t));
      }
    if (e == cudaSuccess)
      e = cudaMallocHost(&G.host_counts, sv->opt.max_batch * sizeof(uint32_t));
    if (e != cudaSuccess)
      return SF_ECUDA;
  }
  std::unique_ptr<SrvSweep> s(new SrvSweep);
  s->bytes = need;
  sf_label_options lo;
  if (label)
    lo = *label;
  else
    sf_default_label_options(&lo);
  s->lab = sf_label_open(height, width, &lo, labeller_capacity(height, width));
  if (!s->lab)
    return SF_EBADARG;
  for (size_t i = 0; i < sv->opt.ring; i++) {
    uint32_t *slot = nullptr;
    if ((e = cudaMalloc(&slot, height * width * sizeof(uint32_t))) != cudaSuccess)
      return SF_ECUDA;
    s->slots.push_back(slot);
    s->free_slots.push_back((int)(sv->opt.ring - 1 - i));
  }
  lock.lock();
  if (fresh) {
    g = fresh.get();
    sv->groups.push_back(std::move(fresh));
    sv->used += gb;
  }
  g->users++;
  s->group = g;
  s->id = sv->next_id++;
  sv->used += need;
  *sweep = s->id;
  sv->sweeps[s->id] = std::move(s);
  return SF_OK;
}

int sf_server_submit(sf_server *sv, int64_t sweep, int64_t frame, const uint32_t *host_frame) {
  if (!sv || !host_frame)
    return SF_EBADARG;
  std::lock_guard<std::mutex> lock(sv->m);
  auto it = sv->sweeps.find(sweep);
  if (it == sv->sweeps.end())
    return SF_EBADARG;
  SrvSweep &s = *it->second;
  // dials_spots.cc:58-63: frames arrive in ascending order.
  if (s.finishing || frame <= s.last_number)
    return SF_EBADARG;
  if (s.status)
    return s.status;
  s.last_number = frame;
  SrvFrame f;
  f.sweep = sweep;
  f.number = frame;
  f.host = host_frame;
  f.t_submit = now_s();
  s.pending.push_back(f);
  s.in_flight++;
  sv->cv_work.notify_all();
  return SF_OK;
}

size_t sf_server_poll(sf_server *sv, sf_frame_done *out, size_t max, int wait_ms) {
  if (!sv || (!out && max))
    return 0;
  std::unique_lock<std::mutex> lock(sv->m);
  if (sv->done.empty() && wait_ms > 0)
    sv->cv_done.wait_for(lock, std::chrono::milliseconds(wait_ms),
                         [&] { return !sv->done.empty(); });
  size_t n = 0;
  while (n < max && !sv->done.empty()) {
    out[n++] = sv->done.front();
    sv->done.pop_front();
  }
  return n;
}

int sf_server_finish_sweep(sf_server *sv, int64_t sweep) {
  if (!sv)
    return SF_EBADARG;
  std::unique_lock<std::mutex> lock(sv->m);
  auto it = sv->sweeps.find(sweep);
  if (it == sv->sweeps.end())
    return SF_EBADARG;
  SrvSweep *s = it->second.get();
  s->finishing = true;
  sv->cv_work.notify_all();
  sv->cv_done.wait(lock, [&] { return s->finished; });
  return s->status;
}

sf_labeller *sf_server_labeller(sf_server *sv, int64_t sweep) {
  if (!sv)
    return nullptr;
  std::lock_guard<std::mutex> lock(sv->m);
  auto it = sv->sweeps.find(sweep);
  return it == sv->sweeps.end() ? nullptr : it->second->lab;
}

int sf_server_close_sweep(sf_server *sv, int64_t sweep) {
  if (!sv)
    return SF_EBADARG;
  std::unique_lock<std::mutex> lock(sv->m);
  auto it = sv->sweeps.find(sweep);
  if (it == sv->sweeps.end())
    return SF_EBADARG;
  SrvSweep *s = it->second.get();
  if (!s->finished) {
    s->finishing = true;
    sv->cv_work.notify_all();
    sv->cv_done.wait(lock, [&] { return s->finished; });
  }
  SrvGroup *g = s->group;
  sv->used -= s->bytes;
  sv->sweeps.erase(it);
  if (--g->users == 0) {
    sv->used -= g->bytes;
    for (auto gi = sv->groups.begin(); gi != sv->groups.end(); ++gi)
      if (gi->get() == g) {
        sv->groups.erase(gi);
        break;
      }
  }
  return SF_OK;
}

size_t sf_server_used_bytes(const sf_server *sv) { return sv ? sv->used : 0; }

} // extern "C"
