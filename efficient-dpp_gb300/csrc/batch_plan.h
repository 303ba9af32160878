// batch_plan.h — host-side plan of the batched kernel (batch.cu), shared with
// the serving loop (host/serve.cpp).  Plain C++: no device code.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "edpp.h"

namespace edpp {

// One segment as the batch kernel reads it.
struct DevSeg {
  int64_t off;     // element offset in the batch arrays
  int64_t state;   // byte offset of the segment's state in the state area
  int32_t len;
  int32_t op;
  int32_t tiles;
  int32_t buckets;
};

// One task: a tile of a segment.
struct DevTask {
  int32_t seg;
  int32_t tile;
  int32_t kind;
  int32_t pad;
};

// Per-segment control words (split: histogram tiles done, ready flag).
struct Ctrl {
  uint32_t hist_done;
  uint32_t ready;
  uint32_t pad[2];
};

struct BatchPlanImpl {
  std::vector<DevSeg> segs;
  // QUEUE schedule: the work queue in order.  KINDS schedule: scan tiles,
  // then gather tiles, then split tiles (one entry per split tile).
  std::vector<DevTask> tasks;
  std::vector<int32_t> split_segs;  // KINDS: segments whose histogram is scanned
  int64_t n_scan = 0, n_gather = 0, n_split = 0;  // KINDS: tiles of each kind
  int64_t queue_tasks = 0;  // tasks of the QUEUE form (a split tile counts twice)
  size_t scan_state_bytes = 0;  // zeroed per launch
  size_t state_bytes = 0;
  size_t off_segs = 0, off_tasks = 0, off_split_segs = 0, off_ctrl = 0, off_state = 0, bytes = 0;
  int num_segs = 0;
  int blocks_per_sm = 4;
  int schedule = 0;  // edpp_batch_schedule
  int64_t total_elems = 0;
};

// Elements per batch tile (every task kind).
constexpr int kBatchTile = 4096;
// Largest bucket count a batch split accepts.
constexpr int kBatchMaxBuckets = 256;

}  // namespace edpp

struct edpp_batch_plan {
  edpp::BatchPlanImpl impl;
};
