// serve.cpp — continuous-batching request loop over the batched kernel.
//
// Clients submit requests (scan / stable split / gather on host arrays) from
// any thread.  One scheduler thread:
//   1. retires finished batches (signalled by a host function enqueued after
//      each batch's device-to-host copies), frees their device memory and
//      completes their requests;
//   2. admits waiting requests in arrival order while device memory in the
//      pool and a batch slot (stream) are free — admission by free HBM;
//   3. packs the admitted requests into one batch: copies their inputs into
//      pool-resident buffers, plans and launches the batch kernels,
//      and copies the outputs back, all stream-ordered on the slot's stream.
// Up to `slots` batches are in flight at once on separate streams, so
// requests that arrive while others run are admitted as memory and slots
// free up and their work overlaps on the device.  Results equal the plain
// calls (bit-exact: all request types are integer).
//
// Device memory: four equal arenas (in0, in1, out0, out1) allocated once at
// creation; a request of n elements holds the same aligned range [o, o+n) in
// all four, so a batch is one edpp_segment table over the arena bases.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch_plan.h"
#include "edpp.h"

namespace {

using Clock = std::chrono::steady_clock;
constexpr int64_t kAlign = 64;  // elements (256 bytes)

int64_t round_up64(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

// First-fit allocator of element ranges with coalescing free list.
class RangeAllocator {
 public:
  explicit RangeAllocator(int64_t capacity) : cap_(capacity) { free_[0] = capacity; }
  // Returns the offset, or -1 if no free range is large enough.
  int64_t alloc(int64_t n) {
    n = round_up64(std::max<int64_t>(n, 1), kAlign);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        const int64_t off = it->first, len = it->second;
        free_.erase(it);
        if (len > n) free_[off + n] = len - n;
        used_ += n;
        return off;
      }
    }
    return -1;
  }
  void release(int64_t off, int64_t n) {
    n = round_up64(std::max<int64_t>(n, 1), kAlign);
    used_ -= n;
    auto it = free_.emplace(off, n).first;
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
      it->second += next->second;
      free_.erase(next);
    }
    if (it != free_.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        free_.erase(it);
      }
    }
  }
  int64_t used() const { return used_; }
  int64_t capacity() const { return cap_; }

 private:
  int64_t cap_;
  int64_t used_ = 0;
  std::map<int64_t, int64_t> free_;
};

struct Request {
  edpp_request req;
  uint64_t id = 0;
  int64_t off = -1;
  Clock::time_point submitted, admitted, done;
  int status = EDPP_OK;
  bool finished = false;
};

struct Slot {
  cudaStream_t stream = nullptr;
  void *ws = nullptr;
  size_t ws_bytes = 0;
  void *staging = nullptr;  // pinned copy of the plan tables
  size_t staging_bytes = 0;
  uint32_t *abort_word = nullptr;  // pinned copy of the batch's abort flag
  bool busy = false;
  std::vector<std::shared_ptr<Request>> reqs;
  std::unique_ptr<edpp_batch_plan, void (*)(edpp_batch_plan *)> plan{nullptr,
                                                                     edpp_batch_plan_destroy};
};

}  // namespace

struct edpp_server {
  edpp_server_config cfg{};
  int device = 0;
  int32_t *arena[4] = {nullptr, nullptr, nullptr, nullptr};
  std::unique_ptr<RangeAllocator> alloc;
  std::vector<Slot> slots;

  std::mutex mu;
  std::condition_variable cv;       // scheduler wake-up
  std::condition_variable done_cv;  // request completion
  std::deque<std::shared_ptr<Request>> pending;
  std::unordered_map<uint64_t, std::shared_ptr<Request>> all;
  std::vector<int> finished_slots;  // filled by host functions
  bool mem_blocked = false;         // the oldest request waits for memory
  uint64_t next_id = 1;
  bool stop = false;
  std::thread thread;
  edpp_server_stats stats{};
};

namespace {

struct SlotDone {
  edpp_server *s;
  int slot;
};

void CUDART_CB on_slot_done(void *arg) {
  // Runs on a CUDA callback thread: no CUDA calls here.
  SlotDone *d = static_cast<SlotDone *>(arg);
  {
    std::lock_guard<std::mutex> lk(d->s->mu);
    d->s->finished_slots.push_back(d->slot);
  }
  d->s->cv.notify_all();
  delete d;
}

// Retire finished batches (lock held).
void retire(edpp_server *s) {
  for (int k : s->finished_slots) {
    Slot &sl = s->slots[static_cast<size_t>(k)];
    // The host function that signalled this slot runs after every earlier
    // operation of the stream completed; the stream itself may still count
    // the host function as running, so "not ready" is not an error here.
    const cudaError_t e = cudaStreamQuery(sl.stream);
    int st = (e == cudaSuccess || e == cudaErrorNotReady) ? EDPP_OK : EDPP_ECUDA;
    if (st == EDPP_OK && *sl.abort_word) st = EDPP_ETIMEOUT;  // a bounded device wait expired
    const auto now = Clock::now();
    for (auto &r : sl.reqs) {
      s->alloc->release(r->off, r->req.length);
      r->done = now;
      r->status = st;
      r->finished = true;
      s->stats.completed++;
      s->stats.elements_done += r->req.length;
    }
    sl.reqs.clear();
    sl.plan.reset();
    sl.busy = false;
  }
  if (!s->finished_slots.empty()) s->done_cv.notify_all();
  s->finished_slots.clear();
}

// Launch one batch of admitted requests on slot k (lock not held).
int launch_batch(edpp_server *s, int k) {
  Slot &sl = s->slots[static_cast<size_t>(k)];
  std::vector<edpp_segment> segs;
  segs.reserve(sl.reqs.size());
  for (auto &r : sl.reqs)
    segs.push_back({r->off, static_cast<int32_t>(r->req.length), r->req.op, r->req.buckets, 0});
  edpp_batch_plan *plan = nullptr;
  int st = edpp_batch_plan_create(segs.data(), static_cast<int>(segs.size()),
                                  &s->cfg.tuning, &plan);
  if (st != EDPP_OK) return st;
  sl.plan.reset(plan);
  const edpp::BatchPlanImpl &p = plan->impl;
  if (p.bytes > sl.ws_bytes) return EDPP_ENOMEM;
  // the plan's tables (segments, tasks, split segment list), as
  // edpp_batch_plan_upload places them, through pinned staging
  const size_t seg_b = sizeof(edpp::DevSeg) * p.segs.size();
  const size_t task_b = sizeof(edpp::DevTask) * p.tasks.size();
  const size_t split_b = sizeof(int32_t) * p.split_segs.size();
  if (seg_b + task_b + split_b > sl.staging_bytes) return EDPP_ENOMEM;
  char *stg = static_cast<char *>(sl.staging);
  std::memcpy(stg, p.segs.data(), seg_b);
  std::memcpy(stg + seg_b, p.tasks.data(), task_b);
  if (split_b) std::memcpy(stg + seg_b + task_b, p.split_segs.data(), split_b);
  char *w = static_cast<char *>(sl.ws);
  cudaStream_t str = sl.stream;
  if (cudaMemcpyAsync(w + p.off_segs, stg, seg_b, cudaMemcpyHostToDevice, str) != cudaSuccess ||
      cudaMemcpyAsync(w + p.off_tasks, stg + seg_b, task_b, cudaMemcpyHostToDevice, str) !=
          cudaSuccess)
    return EDPP_ECUDA;
  if (split_b && cudaMemcpyAsync(w + p.off_split_segs, stg + seg_b + task_b, split_b,
                                 cudaMemcpyHostToDevice, str) != cudaSuccess)
    return EDPP_ECUDA;
  // inputs
  for (auto &r : sl.reqs) {
    const size_t b = sizeof(int32_t) * static_cast<size_t>(r->req.length);
    if (cudaMemcpyAsync(s->arena[0] + r->off, r->req.in0, b, cudaMemcpyHostToDevice, str) !=
        cudaSuccess)
      return EDPP_ECUDA;
    if (r->req.op != EDPP_BATCH_SCAN &&
        cudaMemcpyAsync(s->arena[1] + r->off, r->req.in1, b, cudaMemcpyHostToDevice, str) !=
            cudaSuccess)
      return EDPP_ECUDA;
  }
  st = edpp_batch_launch(plan, s->arena[0], s->arena[1], s->arena[2], s->arena[3], sl.ws,
                         sl.ws_bytes, str);
  if (st != EDPP_OK) return st;
  for (auto &r : sl.reqs) {
    const size_t b = sizeof(int32_t) * static_cast<size_t>(r->req.length);
    if (cudaMemcpyAsync(r->req.out0, s->arena[2] + r->off, b, cudaMemcpyDeviceToHost, str) !=
        cudaSuccess)
      return EDPP_ECUDA;
    if (r->req.op == EDPP_BATCH_SPLIT &&
        cudaMemcpyAsync(r->req.out1, s->arena[3] + r->off, b, cudaMemcpyDeviceToHost, str) !=
            cudaSuccess)
      return EDPP_ECUDA;
  }
  // the batch kernel's abort flag (workspace bytes 8..11) comes back with the outputs
  if (cudaMemcpyAsync(sl.abort_word, w + 8, sizeof(uint32_t), cudaMemcpyDeviceToHost, str) !=
      cudaSuccess)
    return EDPP_ECUDA;
  auto *d = new SlotDone{s, k};
  if (cudaLaunchHostFunc(str, on_slot_done, d) != cudaSuccess) {
    delete d;
    return EDPP_ECUDA;
  }
  return EDPP_OK;
}

void scheduler(edpp_server *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    s->cv.wait(lk, [&] {
      if (s->stop || !s->finished_slots.empty()) return true;
      if (s->pending.empty() || s->mem_blocked) return false;
      for (auto &sl : s->slots)
        if (!sl.busy) return true;
      return false;
    });
    if (!s->finished_slots.empty()) s->mem_blocked = false;
    retire(s);
    bool any_busy = false;
    for (auto &sl : s->slots) any_busy = any_busy || sl.busy;
    if (s->stop && s->pending.empty() && !any_busy) break;
    // admit into one free slot, FIFO, while memory lasts
    int k = -1;
    for (size_t i = 0; i < s->slots.size(); ++i)
      if (!s->slots[i].busy) {
        k = static_cast<int>(i);
        break;
      }
    if (k < 0 || s->pending.empty()) continue;
    Slot &sl = s->slots[static_cast<size_t>(k)];
    int64_t tiles = 0;
    const int64_t max_tiles = s->cfg.max_batch_elements / edpp::kBatchTile + 1;
    while (!s->pending.empty() &&
           static_cast<int>(sl.reqs.size()) < s->cfg.max_batch_requests) {
      auto &r = s->pending.front();
      const int64_t t = (r->req.length + edpp::kBatchTile - 1) / edpp::kBatchTile;
      if (!sl.reqs.empty() && tiles + t > max_tiles) break;
      const int64_t off = s->alloc->alloc(r->req.length);
      if (off < 0) break;  // wait for memory to free up (arrival order kept)
      r->off = off;
      r->admitted = Clock::now();
      tiles += t;
      sl.reqs.push_back(r);
      s->pending.pop_front();
    }
    if (sl.reqs.empty()) {  // the oldest request does not fit until a batch retires
      s->mem_blocked = true;
      continue;
    }
    sl.busy = true;
    s->stats.batches++;
    s->stats.max_requests_per_batch =
        std::max<int64_t>(s->stats.max_requests_per_batch, static_cast<int64_t>(sl.reqs.size()));
    s->stats.max_pool_bytes_used =
        std::max<int64_t>(s->stats.max_pool_bytes_used, 16 * s->alloc->used());
    int inflight = 0;
    for (auto &x : s->slots) inflight += x.busy ? 1 : 0;
    s->stats.max_batches_in_flight = std::max<int64_t>(s->stats.max_batches_in_flight, inflight);
    lk.unlock();
    const int st = launch_batch(s, k);
    lk.lock();
    if (st != EDPP_OK) {  // fail the batch's requests; the slot is freed
      for (auto &r : sl.reqs) {
        s->alloc->release(r->off, r->req.length);
        r->status = st;
        r->finished = true;
        r->done = Clock::now();
      }
      sl.reqs.clear();
      sl.plan.reset();
      sl.busy = false;
      s->done_cv.notify_all();
    }
  }
}

}  // namespace

extern "C" {

int edpp_server_create(const edpp_server_config *cfg, edpp_server **out) {
  if (!cfg || !out || cfg->pool_bytes < (1 << 20) || cfg->slots < 1 || cfg->slots > 16)
    return EDPP_EINVAL;
  auto s = std::unique_ptr<edpp_server>(new (std::nothrow) edpp_server);
  if (!s) return EDPP_ENOMEM;
  s->cfg = *cfg;
  if (s->cfg.max_batch_requests <= 0) s->cfg.max_batch_requests = 1024;
  if (cudaGetDevice(&s->device) != cudaSuccess) return EDPP_ECUDA;
  const int64_t cap = static_cast<int64_t>(cfg->pool_bytes / 16) / kAlign * kAlign;  // elements
  if (s->cfg.max_batch_elements <= 0 || s->cfg.max_batch_elements > cap)
    s->cfg.max_batch_elements = cap;
  s->alloc.reset(new RangeAllocator(cap));
  for (int a = 0; a < 4; ++a)
    if (cudaMalloc(&s->arena[a], static_cast<size_t>(cap) * 4) != cudaSuccess) {
      for (int b = 0; b < a; ++b) cudaFree(s->arena[b]);
      return EDPP_ENOMEM;
    }
  // Workspace per slot: the largest plan a batch can produce (every element
  // of the batch in split segments of the maximum bucket count, and one
  // segment per request).
  const int64_t max_tiles = s->cfg.max_batch_elements / edpp::kBatchTile + s->cfg.max_batch_requests;
  const size_t ws_bytes = 256 + 64 * static_cast<size_t>(s->cfg.max_batch_requests) * 4 +
                          sizeof(edpp::DevTask) * 2 * static_cast<size_t>(max_tiles) +
                          static_cast<size_t>(max_tiles) *
                              (8 + 4 * static_cast<size_t>(edpp::kBatchMaxBuckets)) +
                          256 * static_cast<size_t>(s->cfg.max_batch_requests) * 2 + (1 << 20);
  const size_t staging = (sizeof(edpp::DevSeg) + sizeof(int32_t)) *
                             static_cast<size_t>(s->cfg.max_batch_requests) +
                         sizeof(edpp::DevTask) * 2 * static_cast<size_t>(max_tiles);
  const size_t staging_alloc = staging + 256;  // + the abort word
  s->slots.resize(static_cast<size_t>(cfg->slots));
  for (auto &sl : s->slots) {
    if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&sl.ws, ws_bytes) != cudaSuccess ||
        cudaMallocHost(&sl.staging, staging_alloc) != cudaSuccess) {
      edpp_server_destroy(s.release());
      return EDPP_ENOMEM;
    }
    sl.ws_bytes = ws_bytes;
    sl.staging_bytes = staging;
    sl.abort_word = reinterpret_cast<uint32_t *>(static_cast<char *>(sl.staging) + staging);
    *sl.abort_word = 0;
  }
  edpp_server *raw = s.release();
  raw->thread = std::thread(scheduler, raw);
  *out = raw;
  return EDPP_OK;
}

int edpp_server_submit(edpp_server *s, const edpp_request *req, uint64_t *id) {
  if (!s || !req || !id || req->length < 0 || !req->in0 || !req->out0) return EDPP_EINVAL;
  if (req->op != EDPP_BATCH_SCAN && req->op != EDPP_BATCH_SPLIT && req->op != EDPP_BATCH_GATHER)
    return EDPP_EINVAL;
  if (req->op != EDPP_BATCH_SCAN && !req->in1) return EDPP_EINVAL;
  if (req->op == EDPP_BATCH_SPLIT &&
      (!req->out1 || req->buckets < 1 || req->buckets > edpp::kBatchMaxBuckets ||
       (req->buckets & (req->buckets - 1))))
    return EDPP_EINVAL;
  if (req->length > INT32_MAX || req->length > s->alloc->capacity()) return EDPP_EINVAL;
  auto r = std::make_shared<Request>();
  r->req = *req;
  r->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return EDPP_EINVAL;
    r->id = s->next_id++;
    s->pending.push_back(r);
    s->all[r->id] = r;
    s->stats.submitted++;
  }
  s->cv.notify_all();
  *id = r->id;
  return EDPP_OK;
}

int edpp_server_wait(edpp_server *s, uint64_t id, double timeout_s, edpp_request_timing *timing) {
  if (!s) return EDPP_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return EDPP_EINVAL;
  std::shared_ptr<Request> r = it->second;
  const auto limit = Clock::now() + std::chrono::duration<double>(timeout_s);
  if (!s->done_cv.wait_until(lk, limit, [&] { return r->finished; })) return EDPP_ETIMEOUT;
  if (timing) {
    using ms = std::chrono::duration<double, std::milli>;
    timing->queue_ms = ms(r->admitted - r->submitted).count();
    timing->latency_ms = ms(r->done - r->submitted).count();
  }
  s->all.erase(id);
  return r->status;
}

int edpp_server_get_stats(edpp_server *s, edpp_server_stats *out) {
  if (!s || !out) return EDPP_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  return EDPP_OK;
}

void edpp_server_destroy(edpp_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->thread.joinable()) s->thread.join();
  for (auto &sl : s->slots) {
    if (sl.stream) {
      cudaStreamSynchronize(sl.stream);
      cudaStreamDestroy(sl.stream);
    }
    if (sl.ws) cudaFree(sl.ws);
    if (sl.staging) cudaFreeHost(sl.staging);
  }
  for (auto *a : s->arena)
    if (a) cudaFree(a);
  delete s;
}

}  // extern "C"
