// The served form (include/sf_api.h, sf_server_*): a request loop for frames
// that arrive from several detector streams at once.
//
// Every open sweep keeps its state on the device: a ring of frame slots, the
// signal list of each slot's frame, and its 3-D labeller (the open components
// and their pixels, dials_spots.cc). Sweeps are admitted against a
// device-memory budget. Two kinds of thread run the loop:
//   the worker   copies submitted host frames into the next free slots of
//                their sweep on a copy stream (a compressed chunk is copied
//                and decoded into its slot there), and as soon as frames are on
//                the device forms a batch (continuous batching: whatever is
//                ready across the sweeps of one frame shape and parameter
//                set, up to max_batch), thresholds it in one launch sequence
//                on the compute stream and copies each frame's list into its
//                sweep's slot; it never waits for labelling;
//   one labeller per sweep
//                labels that sweep's frames in frame order on its own stream
//                as their lists become ready; then its frames are done
//                (latency: submit to labelled) and their slots free.
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
#include "sf_decompress.cuh"
#include "sf_label.cuh"

namespace {

// The labellers' streams run at the device's highest priority: a label call
// is a chain of small kernels, each of which would otherwise wait behind a
// whole threshold batch's blocks for an SM, which sets every frame's latency.
int label_priority() {
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return greatest;
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Each frame's list from a batch's outputs into its sweep's slot (which
// holds dst_cap[j] records: the sweep's own capacity, at most the batch's).
struct CopyArgs {
  sf_signal_pixel *dst[SF_MAX_BATCH];
  uint32_t *dst_count[SF_MAX_BATCH];
  size_t dst_cap[SF_MAX_BATCH];
};

__global__ void k_copy_lists(const sf_signal_pixel *__restrict__ src,
                             const uint32_t *__restrict__ counts, size_t capacity,
                             const __grid_constant__ CopyArgs a) {
  const int j = blockIdx.y;
  const uint32_t c = counts[j];
  const size_t cap = capacity < a.dst_cap[j] ? capacity : a.dst_cap[j];
  const size_t n = c < cap ? c : cap;
  const uint4 *s = reinterpret_cast<const uint4 *>(src + (size_t)j * capacity);
  uint4 *d = reinterpret_cast<uint4 *>(a.dst[j]);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    d[i] = s[i];
  if (blockIdx.x == 0 && threadIdx.x == 0)
    *a.dst_count[j] = c;  // an overflowing count stays, and the labeller refuses it
}
static_assert(sizeof(sf_signal_pixel) == sizeof(uint4), "records move as 16 bytes");

struct Event {
  cudaEvent_t e = nullptr;
  Event() { cudaEventCreateWithFlags(&e, cudaEventDisableTiming); }
  ~Event() {
    if (e)
      cudaEventDestroy(e);
  }
};

struct SrvFrame {
  int64_t sweep = 0, number = 0;
  const uint32_t *host = nullptr;
  const uint8_t *chunk = nullptr;        // or a compressed chunk (host)
  std::shared_ptr<sf::ChunkPlan> plan;   // and its blocks
  double t_submit = 0.0;
  int slot = -1;
  std::shared_ptr<Event> up;  // upload (and decode) done
};

// A run of one sweep's frames in consecutive slots, ready once `ready` fires.
struct LabelTask {
  std::vector<SrvFrame> frames;
  int first_slot = 0;
  std::shared_ptr<Event> ready;
};

// Sweeps of one parameter set whose frames fit in the group's shape (the
// shape of the sweep that made it) share launches and outputs: a launch may
// mix detector sizes, laid out for the group's shape.
struct SrvGroup {
  size_t h = 0, w = 0, capacity = 0;
  sf_threshold_params params{};
  void *ws = nullptr;
  size_t ws_bytes = 0;
  sf_signal_pixel *out = nullptr;
  uint32_t *counts = nullptr, *bits = nullptr;
  int users = 0;
  size_t bytes = 0;
  ~SrvGroup() {
    cudaFree(ws);
    cudaFree(out);
    cudaFree(counts);
    cudaFree(bits);
  }
};

struct SrvSweep {
  int64_t id = 0;
  SrvGroup *group = nullptr;
  size_t h = 0, w = 0, capacity = 0;    // its frames' shape, its lists' capacity
  sf_labeller *lab = nullptr;
  size_t bytes = 0, ring = 0;
  size_t result_bytes = 0;              // its labeller's spot and pixel stores, granted
  sf_server *server = nullptr;
  std::vector<uint32_t *> slots;        // frames
  sf_signal_pixel *lists = nullptr;     // ring * capacity records
  uint32_t *counts = nullptr;           // ring
  uint32_t *host_counts = nullptr;      // pinned, ring
  int head = 0;                         // next slot to fill (slots free in order)
  size_t nfree = 0;
  std::deque<SrvFrame> pending;         // submitted, waiting for a slot
  std::deque<SrvFrame> uploaded;        // on the device, waiting for a batch
  std::deque<LabelTask> tasks;          // lists ready (or soon), waiting to be labelled
  size_t in_flight = 0;                 // submitted and not yet done
  int64_t last_number = LLONG_MIN;
  bool finishing = false, finished = false;
  int status = 0;
  std::string error;  // the first failure's message
  std::condition_variable cv;
  std::thread thread;
  cudaStream_t stream = nullptr;
  // Compressed chunks: per slot the decoder's error record (4 words, device
  // and pinned host) and the chunk's block table (device, and the pinned copy
  // it is uploaded from), sized by the first chunk that needs them.
  uint32_t *dec_status = nullptr, *host_dec_status = nullptr;
  std::vector<sf::DecodeBlock *> tables;
  std::vector<void *> host_tables;
  std::vector<size_t> table_bytes;

  void set_error(int rc, const char *why = nullptr) {
    if (status == 0) {
      status = rc;
      const char *m = why ? why : sf_last_error();
      error = m ? m : "";
    }
  }
  ~SrvSweep() {
    if (thread.joinable())
      thread.join();
    if (lab)
      sf_label_close(lab);
    for (uint32_t *p : slots)
      cudaFree(p);
    for (sf::DecodeBlock *p : tables)
      cudaFree(p);
    for (void *p : host_tables)
      if (p)
        cudaFreeHost(p);
    cudaFree(dec_status);
    if (host_dec_status)
      cudaFreeHost(host_dec_status);
    cudaFree(lists);
    cudaFree(counts);
    if (host_counts)
      cudaFreeHost(host_counts);
    if (stream)
      cudaStreamDestroy(stream);
  }
};

// Live pixels a sweep's labeller holds (its open components plus one label
// call's frames): the server's label_capacity, else min(4 Mi, pixels / 2).
size_t labeller_capacity(const sf_server_options &o, size_t h, size_t w) {
  if (o.label_capacity)
    return o.label_capacity;
  return std::min<size_t>((size_t)1 << 22, std::max<size_t>(h * w / 2, 1024));
}

// Device bytes of a labeller of the given capacity (its pools, scratch and
// outputs, as sf_label_open allocates them), with a margin.
size_t labeller_bytes(size_t height, size_t capacity, size_t min_spot_size) {
  return sf::label_device_bytes(height, capacity, min_spot_size) + ((size_t)16 << 20);
}

size_t group_bytes(size_t h, size_t w, size_t capacity, size_t max_batch) {
  const size_t words = (w + 31) / 32 * h;
  return sf_batch_workspace_bytes(max_batch, h, w, capacity) +
         max_batch * (capacity * sizeof(sf_signal_pixel) + words * 4 + 4);
}

bool same_params(const sf_threshold_params &a, const sf_threshold_params &b) {
  return a.algorithm == b.algorithm && a.kernel_x == b.kernel_x && a.kernel_y == b.kernel_y &&
         a.gain == b.gain && a.sigma_b == b.sigma_b && a.sigma_s == b.sigma_s &&
         a.min_local == b.min_local && a.global_threshold == b.global_threshold;
}

} // namespace

struct sf_server {
  sf_server_options opt{};
  int device = 0;
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::map<int64_t, std::unique_ptr<SrvSweep>> sweeps;
  std::vector<std::unique_ptr<SrvGroup>> groups;
  std::deque<sf_frame_done> done;
  std::thread worker;
  bool stop = false;
  int64_t next_id = 1;
  size_t used = 0;
  // Uploads rotate over several copy streams: one stream's copies run one
  // at a time, and the host link needs a few in flight to reach its speed.
  static constexpr int kCopyStreams = 4;
  cudaStream_t copy_s[kCopyStreams] = {}, comp_s = nullptr;
  int next_copy = 0;
  sf_server_stats stats{};
  // Per copy stream, the device copy of the chunk being decoded there (and a
  // scratch frame for bitshuffle blocks over 8 KB); reused in stream order.
  struct DecodeStage {
    uint8_t *chunk = nullptr, *scratch = nullptr;
    size_t chunk_cap = 0, scratch_cap = 0;
  } stage[kCopyStreams];

  bool work_ready() {
    for (auto &kv : sweeps) {
      SrvSweep &s = *kv.second;
      if ((!s.pending.empty() && s.nfree > 0) || !s.uploaded.empty())
        return true;
    }
    return false;
  }

  void run();
  void label_loop(SrvSweep *s);
  cudaError_t upload_chunk(SrvSweep &s, const SrvFrame &f, int ci);
};

// A sweep's results are counted against the budget as its labeller's stores
// grow: a chunk that would take the server past its budget is refused, and
// the sweep fails with SF_EBUSY instead of growing (other sweeps go on).
static bool results_may_grow(void *ctx, size_t bytes) {
  SrvSweep *s = static_cast<SrvSweep *>(ctx);
  sf_server *sv = s->server;
  std::lock_guard<std::mutex> lock(sv->m);
  if (sv->used + bytes > sv->opt.hbm_budget)
    return false;
  sv->used += bytes;
  s->result_bytes += bytes;
  return true;
}

// Copies a frame's chunk to the device on copy stream ci and decodes it into
// the frame's slot there. The slot is free, so its table buffers are idle.
cudaError_t sf_server::upload_chunk(SrvSweep &s, const SrvFrame &f, int ci) {
  const cudaStream_t cs = copy_s[ci];
  const sf::ChunkPlan &p = *f.plan;
  DecodeStage &st = stage[ci];
  cudaError_t e;
  auto grow = [&](uint8_t **buf, size_t *cap, size_t bytes) {
    if (bytes <= *cap)
      return cudaSuccess;
    cudaStreamSynchronize(cs);  // the stream's last decode may still read it
    cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
    const cudaError_t r = cudaMalloc(buf, bytes);
    if (r == cudaSuccess)
      *cap = bytes;
    return r;
  };
  if ((e = grow(&st.chunk, &st.chunk_cap, p.payload)) != cudaSuccess ||
      (p.scratch && (e = grow(&st.scratch, &st.scratch_cap, p.frame_bytes)) != cudaSuccess))
    return e;
  const size_t tb = p.blocks.size() * sizeof(sf::DecodeBlock);
  const int k = f.slot;
  if (tb > s.table_bytes[k]) {
    cudaFree(s.tables[k]);
    if (s.host_tables[k])
      cudaFreeHost(s.host_tables[k]);
    s.tables[k] = nullptr;
    s.host_tables[k] = nullptr;
    s.table_bytes[k] = 0;
    if ((e = cudaMalloc(&s.tables[k], tb)) != cudaSuccess ||
        (e = cudaMallocHost(&s.host_tables[k], tb)) != cudaSuccess)
      return e;
    s.table_bytes[k] = tb;
  }
  std::memcpy(s.host_tables[k], p.blocks.data(), tb);
  if ((e = cudaMemcpyAsync(st.chunk, f.chunk + 12, p.payload, cudaMemcpyHostToDevice, cs)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(s.tables[k], s.host_tables[k], tb, cudaMemcpyHostToDevice, cs)) !=
          cudaSuccess ||
      (e = cudaMemsetAsync(s.dec_status + 4 * k, 0, 4 * sizeof(uint32_t), cs)) != cudaSuccess)
    return e;
  return sf::launch_decode(st.chunk, s.tables[k], p.blocks.size(), p.element,
                           reinterpret_cast<uint8_t *>(s.slots[k]), st.scratch,
                           s.dec_status + 4 * k, s.dec_status + 4 * k + 3, cs);
}

void sf_server::label_loop(SrvSweep *s) {
  cudaSetDevice(device);
  const size_t cap = s->capacity;
  while (true) {
    LabelTask t;
    {
      std::unique_lock<std::mutex> lock(m);
      s->cv.wait(lock, [&] {
        return stop || !s->tasks.empty() || (s->finishing && s->in_flight == 0);
      });
      // A short wait for more of the sweep's frames when the call would be
      // small: a label call has a fixed cost of some forty launches.
      auto queued = [&] {
        size_t n = 0;
        for (const LabelTask &u : s->tasks)
          n += u.frames.size();
        return n;
      };
      if (!stop && !s->finishing && queued() < opt.max_batch)
        s->cv.wait_for(lock, std::chrono::microseconds(opt.coalesce_us), [&] {
          return stop || s->finishing || queued() >= opt.max_batch;
        });
      if (s->tasks.empty()) {
        if (s->finishing && s->in_flight == 0 && !s->finished) {
          const int status = s->status;
          lock.unlock();
          const int rc = status == 0 ? sf_label_finish(s->lab) : status;
          lock.lock();
          if (rc != SF_OK)
            s->set_error(rc);
          s->finished = true;
          cv_done.notify_all();
        }
        if (stop || s->finished)
          return;
        continue;
      }
      // Every waiting run that continues in the next slots joins this call,
      // up to max_batch frames (what the labeller's live pool is sized for):
      // one call's fixed cost for many frames.
      t = std::move(s->tasks.front());
      s->tasks.pop_front();
      cudaStreamWaitEvent(s->stream, t.ready->e, 0);
      while (!s->tasks.empty() &&
             s->tasks.front().first_slot == t.first_slot + (int)t.frames.size() &&
             t.frames.size() + s->tasks.front().frames.size() <= opt.max_batch) {
        LabelTask &u = s->tasks.front();
        cudaStreamWaitEvent(s->stream, u.ready->e, 0);
        for (SrvFrame &f : u.frames)
          t.frames.push_back(f);
        s->tasks.pop_front();
      }
    }
    const size_t k = t.frames.size();
    cudaMemcpyAsync(s->host_counts + t.first_slot, s->counts + t.first_slot,
                    k * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream);
    bool chunks = false;
    for (const SrvFrame &f : t.frames)
      chunks |= f.plan != nullptr;
    if (chunks)
      cudaMemcpyAsync(s->host_dec_status + 4 * t.first_slot, s->dec_status + 4 * t.first_slot,
                      k * 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream);
    int rc = s->status;
    const double t_call = now_s();
    if (rc == SF_OK) {
      std::vector<int64_t> numbers;
      for (const SrvFrame &f : t.frames)
        numbers.push_back(f.number);
      rc = sf_label_add_device(s->lab, numbers.data(), k, s->lists + (size_t)t.first_slot * cap,
                               cap, s->counts + t.first_slot, s->stream);
    }
    cudaStreamSynchronize(s->stream);
    const double now = now_s();
    std::lock_guard<std::mutex> lock(m);
    stats.label_calls++;
    stats.label_frames += k;
    stats.label_seconds += now - t_call;
    stats.label_max_seconds = std::max(stats.label_max_seconds, now - t_call);
    // A chunk the decoder refused fails its frame and the sweep, with the
    // decoder's text (recorded before whatever labelling its frame made of).
    std::vector<int> frc(k, rc);
    for (size_t i = 0; i < k; i++) {
      const uint32_t *dec = s->host_dec_status + 4 * (t.first_slot + i);
      if (t.frames[i].plan && dec[0] != sf::kDecOk) {
        frc[i] = SF_EDATA;
        s->set_error(SF_EDATA, sf::decode_error_text(*t.frames[i].plan, dec).c_str());
      }
    }
    if (rc != SF_OK)
      s->set_error(rc);
    for (size_t i = 0; i < k; i++) {
      sf_frame_done d;
      d.sweep = s->id;
      d.frame = t.frames[i].number;
      d.n_signal = s->host_counts[t.first_slot + i];
      d.status = frc[i];
      d.latency_ms = (now - t.frames[i].t_submit) * 1e3;
      done.push_back(d);
    }
    s->nfree += k;
    s->in_flight -= k;
    cv_done.notify_all();
    cv_work.notify_all();
  }
}

void sf_server::run() {
  cudaSetDevice(device);
  while (true) {
    std::vector<SrvFrame> batch;
    SrvGroup *g = nullptr;
    {
      std::unique_lock<std::mutex> lock(m);
      cv_work.wait(lock, [&] { return stop || work_ready(); });
      if (stop)
        return;
      // A short wait for a fuller batch when few frames are ready.
      auto ready = [&] {
        size_t n = 0;
        for (auto &kv : sweeps)
          n += kv.second->uploaded.size() + std::min(kv.second->pending.size(), kv.second->nfree);
        return n;
      };
      if (ready() < opt.max_batch)
        cv_work.wait_for(lock, std::chrono::microseconds(opt.coalesce_us),
                         [&] { return stop || ready() >= opt.max_batch; });
      // 1. Uploads into the sweeps' next slots, in submission order.
      for (auto &kv : sweeps) {
        SrvSweep &s = *kv.second;
        while (!s.pending.empty() && s.nfree > 0) {
          SrvFrame f = s.pending.front();
          s.pending.pop_front();
          f.slot = s.head;
          s.head = (s.head + 1) % (int)s.ring;
          s.nfree--;
          f.up = std::make_shared<Event>();
          const size_t bytes = s.h * s.w * sizeof(uint32_t);
          const int ci = next_copy;
          const cudaStream_t cs = copy_s[ci];
          next_copy = (next_copy + 1) % kCopyStreams;
          cudaError_t e = f.plan ? upload_chunk(s, f, ci)
                                 : cudaMemcpyAsync(s.slots[f.slot], f.host, bytes,
                                                   cudaMemcpyHostToDevice, cs);
          if (e == cudaSuccess)
            e = cudaEventRecord(f.up->e, cs);
          if (e != cudaSuccess)
            s.set_error(SF_ECUDA, "copying a frame to the device");
          s.uploaded.push_back(f);
        }
      }
      // 2. A batch: the shape group of the oldest frame on the device, every
      // ready frame of its sweeps up to max_batch, grouped by sweep in order.
      SrvSweep *first = nullptr;
      for (auto &kv : sweeps) {
        SrvSweep &s = *kv.second;
        if (!s.uploaded.empty() &&
            (!first || s.uploaded.front().t_submit < first->uploaded.front().t_submit))
          first = &s;
      }
      if (!first)
        continue;
      g = first->group;
      for (auto &kv : sweeps) {
        SrvSweep &s = *kv.second;
        if (s.group != g)
          continue;
        while (!s.uploaded.empty() && batch.size() < opt.max_batch) {
          batch.push_back(s.uploaded.front());
          s.uploaded.pop_front();
        }
      }
    }
    // 3. Threshold the batch, then each list into its sweep's slot.
    const double t_launch = now_s();
    std::vector<const uint32_t *> images;
    std::vector<size_t> heights, widths;
    CopyArgs ca;
    {
      std::lock_guard<std::mutex> lock(m);
      for (size_t j = 0; j < batch.size(); j++) {
        SrvSweep &s = *sweeps[batch[j].sweep];
        images.push_back(s.slots[batch[j].slot]);
        heights.push_back(s.h);
        widths.push_back(s.w);
        ca.dst[j] = s.lists + (size_t)batch[j].slot * s.capacity;
        ca.dst_count[j] = s.counts + batch[j].slot;
        ca.dst_cap[j] = s.capacity;
      }
    }
    for (SrvFrame &f : batch)
      cudaStreamWaitEvent(comp_s, f.up->e, 0);
    // One launch sequence for the batch, whatever detector sizes it mixes.
    const int rc = sf_threshold_u32_mixed_batch_device(
        images.data(), heights.data(), widths.data(), images.size(), &g->params, g->out,
        g->capacity, g->bits, g->counts, nullptr, g->ws, g->ws_bytes, comp_s);
    if (rc == SF_OK)
      k_copy_lists<<<dim3(8, (unsigned)batch.size()), 256, 0, comp_s>>>(g->out, g->counts,
                                                                       g->capacity, ca);
    auto ready = std::make_shared<Event>();
    cudaEventRecord(ready->e, comp_s);
    // 4. Each sweep's run of frames goes to its labeller, split where its
    // slots wrap (a label call takes evenly spaced lists).
    std::lock_guard<std::mutex> lock(m);
    stats.batches++;
    stats.batch_frames += batch.size();
    const double launch_s = now_s() - t_launch;
    stats.launch_seconds += launch_s;
    stats.launch_max_seconds = std::max(stats.launch_max_seconds, launch_s);
    size_t j = 0;
    while (j < batch.size()) {
      SrvSweep &s = *sweeps[batch[j].sweep];
      if (rc != SF_OK)
        s.set_error(rc);
      LabelTask t;
      t.first_slot = batch[j].slot;
      t.ready = ready;
      while (j < batch.size() && batch[j].sweep == s.id &&
             batch[j].slot == t.first_slot + (int)t.frames.size()) {
        batch[j].up.reset();
        t.frames.push_back(batch[j]);
        j++;
      }
      s.tasks.push_back(std::move(t));
      s.cv.notify_all();
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
  o->coalesce_us = 1000;
  o->label_capacity = 0;
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
  bool ok = cudaStreamCreateWithFlags(&sv->comp_s, cudaStreamNonBlocking) == cudaSuccess;
  for (cudaStream_t &cs : sv->copy_s)
    ok = ok && cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess;
  if (!ok) {
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
    for (auto &kv : sv->sweeps)
      kv.second->cv.notify_all();
  }
  sv->cv_work.notify_all();
  if (sv->worker.joinable())
    sv->worker.join();
  for (auto &kv : sv->sweeps)
    if (kv.second->thread.joinable())
      kv.second->thread.join();
  cudaDeviceSynchronize();
  sv->sweeps.clear();
  sv->groups.clear();
  for (auto &st : sv->stage) {
    cudaFree(st.chunk);
    cudaFree(st.scratch);
  }
  for (cudaStream_t cs : sv->copy_s)
    cudaStreamDestroy(cs);
  cudaStreamDestroy(sv->comp_s);
  delete sv;
}

size_t sf_server_sweep_bytes(const sf_server *sv, size_t height, size_t width,
                             const sf_label_options *label) {
  if (!sv || height == 0 || width == 0)
    return 0;
  const size_t min_size = label ? label->min_spot_size : 3;
  const size_t capacity = std::max<size_t>(1, height * width / sv->opt.capacity_divisor);
  return sv->opt.ring * (height * width * sizeof(uint32_t) + capacity * sizeof(sf_signal_pixel) +
                         sizeof(uint32_t)) +
         labeller_bytes(height, labeller_capacity(sv->opt, height, width), min_size);
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
    if (!g && height <= gr->h && width <= gr->w && same_params(gr->params, p))
      g = gr.get();
  const size_t need = sf_server_sweep_bytes(sv, height, width, label);
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
    if ((e = cudaMalloc(&G.ws, G.ws_bytes)) == cudaSuccess &&
        (e = cudaMalloc(&G.out, sv->opt.max_batch * capacity * sizeof(sf_signal_pixel))) ==
            cudaSuccess &&
        (e = cudaMalloc(&G.counts, sv->opt.max_batch * sizeof(uint32_t))) == cudaSuccess)
      e = cudaMalloc(&G.bits, sv->opt.max_batch * words * sizeof(uint32_t));
    if (e != cudaSuccess)
      return SF_ECUDA;
  }
  std::unique_ptr<SrvSweep> s(new SrvSweep);
  s->h = height;
  s->w = width;
  s->capacity = capacity;
  s->bytes = need;
  s->ring = sv->opt.ring;
  s->nfree = s->ring;
  sf_label_options lo;
  if (label)
    lo = *label;
  else
    sf_default_label_options(&lo);
  s->lab = sf_label_open(height, width, &lo, labeller_capacity(sv->opt, height, width));
  if (!s->lab)
    return SF_EBADARG;
  s->server = sv;
  sf::LabelGrowth growth;
  growth.ok = results_may_grow;
  growth.ctx = s.get();
  sf::label_set_growth(s->lab, growth);
  // Its label thread sleeps while a call runs, and every call shape is
  // captured now rather than in the middle of the sweep's frames.
  int lrc = sf::label_set_blocking_wait(s->lab);
  if (lrc == SF_OK)
    lrc = sf::label_prepare(s->lab, (int)sv->opt.max_batch);
  if (lrc != SF_OK)
    return lrc;
  for (size_t i = 0; i < s->ring; i++) {
    uint32_t *slot = nullptr;
    if ((e = cudaMalloc(&slot, height * width * sizeof(uint32_t))) != cudaSuccess)
      return SF_ECUDA;
    s->slots.push_back(slot);
  }
  s->tables.assign(s->ring, nullptr);
  s->host_tables.assign(s->ring, nullptr);
  s->table_bytes.assign(s->ring, 0);
  if ((e = cudaMalloc(&s->lists, s->ring * capacity * sizeof(sf_signal_pixel))) != cudaSuccess ||
      (e = cudaMalloc(&s->counts, s->ring * sizeof(uint32_t))) != cudaSuccess ||
      (e = cudaMallocHost(&s->host_counts, s->ring * sizeof(uint32_t))) != cudaSuccess ||
      (e = cudaMalloc(&s->dec_status, s->ring * 4 * sizeof(uint32_t))) != cudaSuccess ||
      (e = cudaMallocHost(&s->host_dec_status, s->ring * 4 * sizeof(uint32_t))) != cudaSuccess ||
      (e = cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking, label_priority())) !=
          cudaSuccess)
    return SF_ECUDA;
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
  SrvSweep *raw = s.get();
  sv->sweeps[s->id] = std::move(s);
  raw->thread = std::thread([sv, raw] { sv->label_loop(raw); });
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

int sf_server_submit_chunk(sf_server *sv, int64_t sweep, int64_t frame, const uint8_t *data,
                           size_t nbytes, const char *algorithm) {
  if (!sv || !data)
    return SF_EBADARG;
  size_t h = 0, w = 0;
  {
    std::lock_guard<std::mutex> lock(sv->m);
    auto it = sv->sweeps.find(sweep);
    if (it == sv->sweeps.end())
      return SF_EBADARG;
    h = it->second->h;
    w = it->second->w;
  }
  // The chunk's header and framing, checked before the frame is taken
  // (decompress.cc:77-134), off the lock.
  auto plan = std::make_shared<sf::ChunkPlan>();
  const int rc = sf::plan_chunk(data, nbytes, algorithm, 32, h, w, h * w * sizeof(uint32_t),
                                plan.get());
  if (rc != SF_OK)
    return rc;
  if (plan->algorithm == sf::kChunkNone)
    return sf_server_submit(sv, sweep, frame, reinterpret_cast<const uint32_t *>(data));
  std::lock_guard<std::mutex> lock(sv->m);
  auto it = sv->sweeps.find(sweep);
  if (it == sv->sweeps.end())
    return SF_EBADARG;
  SrvSweep &s = *it->second;
  if (s.finishing || frame <= s.last_number)
    return SF_EBADARG;
  if (s.status)
    return s.status;
  s.last_number = frame;
  SrvFrame f;
  f.sweep = sweep;
  f.number = frame;
  f.chunk = data;
  f.plan = std::move(plan);
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

static int wait_finished(sf_server *sv, std::unique_lock<std::mutex> &lock, SrvSweep *s) {
  s->finishing = true;
  s->cv.notify_all();
  sv->cv_work.notify_all();
  // Bounded: a sweep whose frames never complete reports an error rather
  // than holding the caller.
  if (!sv->cv_done.wait_for(lock, std::chrono::seconds(120), [&] { return s->finished; })) {
    s->set_error(SF_ECUDA, "finishing a sweep timed out");
    return SF_ECUDA;
  }
  return s->status;
}

int sf_server_finish_sweep(sf_server *sv, int64_t sweep) {
  if (!sv)
    return SF_EBADARG;
  std::unique_lock<std::mutex> lock(sv->m);
  auto it = sv->sweeps.find(sweep);
  if (it == sv->sweeps.end())
    return SF_EBADARG;
  return wait_finished(sv, lock, it->second.get());
}

sf_labeller *sf_server_labeller(sf_server *sv, int64_t sweep) {
  if (!sv)
    return nullptr;
  std::lock_guard<std::mutex> lock(sv->m);
  auto it = sv->sweeps.find(sweep);
  return it == sv->sweeps.end() ? nullptr : it->second->lab;
}

const char *sf_server_sweep_error(sf_server *sv, int64_t sweep) {
  if (!sv)
    return "";
  std::lock_guard<std::mutex> lock(sv->m);
  auto it = sv->sweeps.find(sweep);
  return it == sv->sweeps.end() ? "" : it->second->error.c_str();
}

int sf_server_close_sweep(sf_server *sv, int64_t sweep) {
  if (!sv)
    return SF_EBADARG;
  std::unique_lock<std::mutex> lock(sv->m);
  auto it = sv->sweeps.find(sweep);
  if (it == sv->sweeps.end())
    return SF_EBADARG;
  SrvSweep *s = it->second.get();
  if (!s->finished && wait_finished(sv, lock, s) == SF_ECUDA && !s->finished)
    return SF_ECUDA;
  std::unique_ptr<SrvSweep> gone = std::move(it->second);
  sv->sweeps.erase(it);
  SrvGroup *g = gone->group;
  sv->used -= gone->bytes + gone->result_bytes;
  std::unique_ptr<SrvGroup> gone_group;
  if (--g->users == 0) {
    sv->used -= g->bytes;
    for (auto gi = sv->groups.begin(); gi != sv->groups.end(); ++gi)
      if (gi->get() == g) {
        gone_group = std::move(*gi);
        sv->groups.erase(gi);
        break;
      }
  }
  lock.unlock();
  gone.reset();  // joins its (finished) label thread, frees its memory
  return SF_OK;
}

size_t sf_server_used_bytes(const sf_server *sv) { return sv ? sv->used : 0; }

void sf_server_get_stats(sf_server *sv, sf_server_stats *out) {
  if (!sv || !out)
    return;
  std::lock_guard<std::mutex> lock(sv->m);
  *out = sv->stats;
}

} // extern "C"
