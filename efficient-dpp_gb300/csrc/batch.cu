// batch.cu — many uneven segments of scan / stable split / permutation gather
// from one uploaded plan, in a handful of launches.
//
// The host planner (below) cuts every segment into tiles of kTile elements.
// Tile kinds:
//   SCAN     exclusive int32 scan tile; tiles of a segment are chained by a
//            decoupled look-back over the segment's own tile states
//   GATHER   out0[i] = in0[in1[i]] for a tile, indices local to the segment
//   HIST     bucket counts of a split tile -> column t of the segment's
//            bucket-major histogram his[b*T + t]
//   SPLIT    stable key/value scatter of a tile once the segment's histogram
//            is scanned; same ranking as split.cu, 64-bucket-class tiles
//
// Two schedules (edpp_batch_tuning.schedule):
//   KINDS  one launch per kind, one block per tile: scan tiles, gather tiles,
//          HIST tiles, one block per split segment scanning its histogram,
//          SPLIT tiles.  Stream order separates the kinds; a scan tile waits
//          only on lower tiles of its segment (lower block indices).
//   QUEUE  one persistent kernel; blocks take tasks from one atomic ticket in
//          queue order.  The block that finishes a segment's last HIST tile
//          scans the histogram and publishes a ready flag (release) that the
//          SPLIT tiles acquire.  A task waits only on tasks earlier in the
//          queue, which running blocks already hold, so the schedule always
//          makes progress.  Knobs (chosen per size class by
//          edpp_batch_autotune): blocks per SM, how many segments a split's
//          SPLIT tasks trail its HIST tasks, and the segment order.
// Every wait is bounded by %globaltimer and reports EDPP_FAULT_TIMEOUT
// instead of hanging.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <numeric>
#include <vector>

#include "batch_plan.h"
#include "scan_tile.cuh"

namespace edpp {
namespace {

constexpr int kThreads = 256;
constexpr int kChunks = 4;
using TS32 = TileScan<int32_t, kThreads, kChunks>;
constexpr int kTile = TS32::kTile;  // 4096 elements for every task kind
static_assert(kTile == kBatchTile, "batch tile size");
constexpr int kWarps = kThreads / 32;
constexpr int kSeg = kTile / kWarps;  // 512 elements per warp in SPLIT
constexpr int kIters = kSeg / 32;     // 16
constexpr int kMaxB = kBatchMaxBuckets;

enum TaskKind : int32_t { kTaskScan = 0, kTaskGather = 1, kTaskHist = 2, kTaskSplit = 3 };

__device__ __forceinline__ unsigned lanemask_lt_b() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

union __align__(128) BatchSmem {
  struct {
    int32_t tile[kTile];
    TS32::Shared sh;
  } scan;
  struct {
    int32_t keys[kTile];  // with vals: the tile as loaded; re-laid out, {key, value} pairs
    int32_t vals[kTile];
    uint16_t cnt16[kWarps * kMaxB];
    int32_t gofs[kMaxB];
    uint32_t peer[kWarps * kMaxB];  // lanes of each (warp, bucket), ORed in by rank round
  } split;
  struct {
    uint32_t cnt[kMaxB];
    int32_t wsum[32];
  } hist;
};

// Exclusive scan of p[0..m) in place by the whole block (m up to millions),
// in rounds of kThreads x 4 consecutive elements (p 16-byte aligned: one
// vector per thread), carrying the running total between rounds.
__device__ void block_exclusive_scan_inplace(int32_t *p, int64_t m, int32_t *wsum) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  constexpr int kRound = kThreads * 4;
  uint32_t carry = 0;
  for (int64_t base = 0; base < m; base += kRound) {
    const int64_t i0 = base + 4 * t;
    uint32_t v[4] = {0u, 0u, 0u, 0u};
    if (i0 + 3 < m) {
      const int4 q = __ldcg(reinterpret_cast<const int4 *>(p + i0));
      v[0] = static_cast<uint32_t>(q.x), v[1] = static_cast<uint32_t>(q.y);
      v[2] = static_cast<uint32_t>(q.z), v[3] = static_cast<uint32_t>(q.w);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (i0 + k < m) v[k] = static_cast<uint32_t>(__ldcg(p + i0 + k));
    }
    const uint32_t s = v[0] + v[1] + v[2] + v[3];
    uint32_t incl = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += y;
    }
    if (lane == 31) wsum[w] = static_cast<int32_t>(incl);
    __syncthreads();
    uint32_t wpre = 0, total = 0;
#pragma unroll
    for (int k = 0; k < kWarps; ++k) {
      const uint32_t x = static_cast<uint32_t>(wsum[k]);
      if (k < w) wpre += x;
      total += x;
    }
    uint32_t run = carry + wpre + (incl - s);
    if (i0 + 3 < m) {
      int4 q;
      q.x = static_cast<int32_t>(run);
      q.y = static_cast<int32_t>(run += v[0]);
      q.z = static_cast<int32_t>(run += v[1]);
      q.w = static_cast<int32_t>(run += v[2]);
      *reinterpret_cast<int4 *>(p + i0) = q;
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (i0 + k < m) {
          p[i0 + k] = static_cast<int32_t>(run);
          run += v[k];
        }
    }
    carry += total;
    __syncthreads();  // wsum is rewritten by the next round
  }
}

// ---- tile task bodies, shared by the work-queue kernel and the per-kind kernels ----

struct TaskIO {
  const int32_t *in0, *in1;
  int32_t *out0, *out1;
  char *state;
  uint64_t timeout_ns;
  unsigned *fault, *abort_flag;
  bool tma;   // in0 16-byte aligned
  bool tma1;  // in1 16-byte aligned
  int num_segs;
};

// A task's segment and tile must lie inside the plan's tables (a workspace
// without an uploaded plan holds garbage): otherwise record EDPP_FAULT_PLAN
// and skip the task.  Block-uniform.
__device__ __forceinline__ bool task_in_plan(const DevTask &task, const DevSeg *segs,
                                             const TaskIO &io, DevSeg &seg) {
  if (task.seg < 0 || task.seg >= io.num_segs) {
    if (threadIdx.x == 0) raise_fault(io.fault, EDPP_FAULT_PLAN);
    return false;
  }
  seg = segs[task.seg];
  if (task.tile < 0 || task.tile >= seg.tiles) {
    if (threadIdx.x == 0) raise_fault(io.fault, EDPP_FAULT_PLAN);
    return false;
  }
  return true;
}

// Exclusive scan of one tile with a decoupled look-back over the segment's
// own tile states.  `released()` runs (every thread) once no other task can
// wait on this one any more: after the inclusive prefix is published.
template <typename TS, int NT, int CHUNKS, typename F>
__device__ __forceinline__ void scan_tile_task(const DevSeg &seg, int tile, const TaskIO &io,
                                               int32_t *tile_smem, typename TS::Shared &sh,
                                               uint64_t *bar, uint32_t &phase, F released) {
  static_assert(TS::kTile == kTile, "batch tile size");
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int64_t tile_base = static_cast<int64_t>(tile) * kTile;
  const int count = static_cast<int>(min64(kTile, seg.len - tile_base));
  const int64_t gbase = seg.off + tile_base;
  LookbackState<int32_t> st;
  st.bind(io.state + seg.state, seg.tiles);
  const bool tma_ok = io.tma && ((gbase & 3) == 0);  // 16-byte aligned tile start
  const uint32_t bulk =
      stage_tile<int32_t, kTile, NT>(tile_smem, io.in0 + gbase, count, tma_ok, bar);
  if (bulk) {
    if (!mbar_wait_bounded(bar, phase, io.timeout_ns, io.fault)) atomicOr(io.abort_flag, 1u);
    phase ^= 1u;
  }
  __syncthreads();
  Chunk<int32_t> c[CHUNKS];
  int32_t wex[CHUNKS];
  TS::phase1(tile_smem, c, wex, sh);
  __syncthreads();
  if (w == 0) {
    const int32_t agg = TS::phase2_warp0(sh, lane);
    int32_t prefix = 0;
    bool ok = true;
    if (tile == 0) {
      if (lane == 0) st.publish(0, kFlagIncl, agg);
    } else {
      prefix = lookback_warp<int32_t>(st, tile, agg, lane, io.timeout_ns, io.fault, io.abort_flag,
                                      ok);
    }
    if (lane == 0) sh.prefix = ok ? prefix : 0;
  }
  released();
  __syncthreads();
  TS::template phase3<false>(c, wex, sh, sh.prefix);
  TS::store(io.out0, gbase, count, c, (reinterpret_cast<uintptr_t>(io.out0 + gbase) & 15) == 0);
}

// Permutation gather of one tile, indices local to the segment.
__device__ __forceinline__ void gather_tile_task(const DevSeg &seg, int tile, const TaskIO &io) {
  const int t = threadIdx.x;
  const int64_t tile_base = static_cast<int64_t>(tile) * kTile;
  const int count = static_cast<int>(min64(kTile, seg.len - tile_base));
  const int64_t gbase = seg.off + tile_base;
  const int32_t *src = io.in0 + seg.off;
#pragma unroll
  for (int k = 0; k < kTile / kThreads; k += 4) {
    int v[4], idx[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = (k + q) * kThreads + t;
      idx[q] = i < count ? io.in1[gbase + i] : -1;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = (idx[q] >= 0 && idx[q] < seg.len) ? src[idx[q]] : 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = (k + q) * kThreads + t;
      if (idx[q] >= 0 && idx[q] < seg.len) io.out0[gbase + i] = v[q];
    }
  }
}

// Bucket counts of one split tile -> column `tile` of the segment's
// bucket-major histogram his[b*T + tile].  cnt: shared, >= seg.buckets.
__device__ __forceinline__ void hist_tile_task(const DevSeg &seg, int tile, const TaskIO &io,
                                               uint32_t *cnt) {
  const int t = threadIdx.x;
  const int64_t tile_base = static_cast<int64_t>(tile) * kTile;
  const int count = static_cast<int>(min64(kTile, seg.len - tile_base));
  const int64_t gbase = seg.off + tile_base;
  const unsigned mask = static_cast<unsigned>(seg.buckets - 1);
  // all of this thread's keys are loaded before the first count
  int32_t k[kTile / kThreads];
  const int32_t *src = io.in0 + gbase;
  if (count == kTile && io.tma && (gbase & 3) == 0) {  // 16-byte aligned full tile
#pragma unroll
    for (int q = 0; q < kTile / kThreads / 4; ++q) {
      const int4 v = __ldcs(reinterpret_cast<const int4 *>(src) + q * kThreads + t);
      k[4 * q] = v.x, k[4 * q + 1] = v.y, k[4 * q + 2] = v.z, k[4 * q + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int q = 0; q < kTile / kThreads / 4; ++q)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = 4 * (q * kThreads + t) + e;
        k[4 * q + e] = i < count ? src[i] : 0;
      }
  }
  for (int b = t; b < seg.buckets; b += kThreads) cnt[b] = 0;
  __syncthreads();
#pragma unroll
  for (int q = 0; q < kTile / kThreads / 4; ++q)
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (4 * (q * kThreads + t) + e < count)
        atomicAdd(&cnt[static_cast<unsigned>(k[4 * q + e]) & mask], 1u);
  __syncthreads();
  int32_t *his = reinterpret_cast<int32_t *>(io.state + seg.state);
  for (int b = t; b < seg.buckets; b += kThreads)
    his[static_cast<int64_t>(b) * seg.tiles + tile] = static_cast<int32_t>(cnt[b]);
}

// Stable key/value scatter of one split tile; the segment's histogram is
// scanned (his[b*T + t] = first output index of bucket b from tile t).
// Ranks as in split.cu, with 16-bit shared counters per (warp, bucket):
// votes on the bucket bits up to 8 buckets (kMask false), per-warp lane
// masks above.  The tile comes in by bulk copies (its
// 16-byte-aligned part) on `bar`; warp 0 loads the tile's first 64 run
// starts before the ranking, so that round trip overlaps it.
constexpr int kHisPre = 2;  // run starts per lane of warp 0 loaded early
template <bool kMask>
__device__ __forceinline__ void split_tile_run(const DevSeg &seg, int tile, const TaskIO &io,
                                               BatchSmem &sm, uint64_t *bar, uint32_t &phase) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const unsigned lt = lanemask_lt_b();
  const int64_t tile_base = static_cast<int64_t>(tile) * kTile;
  const int count = static_cast<int>(min64(kTile, seg.len - tile_base));
  const int64_t gbase = seg.off + tile_base;
  const unsigned mask = static_cast<unsigned>(seg.buckets - 1);
  const int B = seg.buckets;
  const int32_t *his = reinterpret_cast<const int32_t *>(io.state + seg.state);
  const uint32_t bulk =
      (io.tma && io.tma1 && (gbase & 3) == 0) ? (static_cast<uint32_t>(count) * 4u) & ~15u : 0u;
  if (t == 0 && bulk) {
    mbar_arrive_expect_tx(bar, 2 * bulk);
    tma_load_1d(sm.split.keys, io.in0 + gbase, bulk, bar);
    tma_load_1d(sm.split.vals, io.in1 + gbase, bulk, bar);
  }
  for (int i = static_cast<int>(bulk / 4) + t; i < count; i += kThreads) {
    sm.split.keys[i] = io.in0[gbase + i];
    sm.split.vals[i] = io.in1[gbase + i];
  }
  int32_t his_pre[kHisPre] = {0, 0};
  if (w == 0) {
#pragma unroll
    for (int j = 0; j < kHisPre; ++j) {
      const int b = j * 32 + lane;
      if (b < B) his_pre[j] = __ldcg(his + static_cast<int64_t>(b) * seg.tiles + tile);
    }
  }
  for (int i = t; i < kWarps * B; i += kThreads) {
    sm.split.cnt16[i] = 0;
    if (kMask) sm.split.peer[i] = 0u;
  }
  if (bulk) {
    if (!mbar_wait_bounded(bar, phase, io.timeout_ns, io.fault)) atomicOr(io.abort_flag, 1u);
    phase ^= 1u;
  }
  __syncthreads();
  uint16_t *my = sm.split.cnt16 + w * B;
  const int kbits = 31 - __clz(B);
  int32_t kk[kIters], vv[kIters];
  uint32_t rk[kIters / 2];
#pragma unroll
  for (int it = 0; it < kIters; ++it) {
    const int pos = w * kSeg + it * 32 + lane;
    const bool valid = pos < count;
    const int32_t key = valid ? sm.split.keys[pos] : 0;
    const int32_t val = valid ? sm.split.vals[pos] : 0;
    const int b = valid ? static_cast<int>(static_cast<unsigned>(key) & mask) : -1;
    const unsigned vmask = __ballot_sync(0xffffffffu, valid);
    unsigned peers;
    if (!kMask) {
      peers = match_low_bits(static_cast<unsigned>(b), kbits, vmask);
    } else {  // each lane ORs its bit into its bucket's mask and reads the group back
      if (valid) atomicOr(&sm.split.peer[w * B + b], 1u << lane);
      __syncwarp();
      peers = valid ? sm.split.peer[w * B + b] : 0u;
    }
    const unsigned lower = peers & lt;
    const uint16_t before = valid ? my[b] : 0;
    __syncwarp();
    if (valid && lower == 0u) {
      my[b] = static_cast<uint16_t>(before + __popc(peers));
      if (kMask) sm.split.peer[w * B + b] = 0u;
    }
    __syncwarp();
    kk[it] = key;
    vv[it] = val;
    const uint32_t r = static_cast<uint32_t>(before + __popc(lower));
    if (it & 1) rk[it >> 1] |= r << 16;
    else rk[it >> 1] = r;
  }
  __syncthreads();
  // per bucket: tile count, tile offset, then each warp's first slot
  // (cnt16[w][b] becomes the bucket's tile offset plus the counts of the
  // warps before w, so the re-layout looks up one counter per element)
  if (t < 32) {
    int32_t run_total = 0;
    for (int b0 = 0; b0 < B; b0 += 32) {
      const int b = b0 + lane;
      int32_t tot = 0;
      if (b < B)
        for (int ww = 0; ww < kWarps; ++ww) tot += sm.split.cnt16[ww * B + b];
      int32_t incl = tot;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
      }
      if (b < B) {
        const int32_t off = run_total + incl - tot;
        int32_t slot = off;
        for (int ww = 0; ww < kWarps; ++ww) {
          const int32_t c = sm.split.cnt16[ww * B + b];
          sm.split.cnt16[ww * B + b] = static_cast<uint16_t>(slot);
          slot += c;
        }
        const int j = b0 / 32;
        const int32_t start = j == 0   ? his_pre[0]
                              : j == 1 ? his_pre[1]
                                       : __ldcg(his + static_cast<int64_t>(b) * seg.tiles + tile);
        sm.split.gofs[b] = start - off;
      }
      run_total += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < kIters; ++it) {
    const int pos = w * kSeg + it * 32 + lane;
    if (pos < count) {
      const int b = static_cast<int>(static_cast<unsigned>(kk[it]) & mask);
      const int r = static_cast<int>((rk[it >> 1] >> ((it & 1) * 16)) & 0xffffu);
      const int s = sm.split.cnt16[w * B + b] + r;
      reinterpret_cast<int2 *>(sm.split.keys)[s] = make_int2(kk[it], vv[it]);
    }
  }
  __syncthreads();
  for (int s = t; s < count; s += kThreads) {
    const int2 kv = reinterpret_cast<const int2 *>(sm.split.keys)[s];
    const int32_t key = kv.x;
    const int b = static_cast<int>(static_cast<unsigned>(key) & mask);
    const int64_t o = seg.off + sm.split.gofs[b] + s;
    io.out0[o] = key;
    io.out1[o] = kv.y;
  }
}

// Ranking form chosen once per tile (votes up to 8 buckets, lane masks
// above), so each form's unrolled loop is compiled on its own.
__device__ __forceinline__ void split_tile_task(const DevSeg &seg, int tile, const TaskIO &io,
                                                BatchSmem &sm, uint64_t *bar, uint32_t &phase) {
  if (seg.buckets > 8) split_tile_run<true>(seg, tile, io, sm, bar, phase);
  else split_tile_run<false>(seg, tile, io, sm, bar, phase);
}

// ---- QUEUE schedule: one persistent launch over the work queue ----
__global__ void __launch_bounds__(kThreads, 3)
    batch_kernel(const DevSeg *__restrict__ segs, const DevTask *__restrict__ tasks, int num_tasks,
                 TaskIO io, Ctrl *ctrl, unsigned long long *ticket) {
  __shared__ BatchSmem sm;
  __shared__ alignas(8) uint64_t bar;
  __shared__ int s_task;
  __shared__ int s_flag;
  const int t = threadIdx.x;
  if (t == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t phase = 0;

  // Thread 0 takes the next ticket early, once nothing can wait on the
  // current task any more: a SCAN tile after publishing its prefix, a SPLIT
  // tile once its histogram is ready, a GATHER tile at once (HIST tiles take
  // it at the loop top).  The atomic's latency then hides behind the rest of
  // the task, and a block never holds an unstarted task while the current one
  // can still make others wait, so waits do not chain.
  int next_task = -1;
  auto take_next = [&]() {
    if (t == 0 && next_task < 0) next_task = static_cast<int>(atomicAdd(ticket, 1ull));
  };

  while (true) {
    if (t == 0) {
      take_next();
      s_task = next_task;
      next_task = -1;
    }
    __syncthreads();
    const int task_id = s_task;
    if (task_id >= num_tasks) break;
    const DevTask task = tasks[task_id];
    DevSeg seg;
    if (!task_in_plan(task, segs, io, seg)) {
      if (t == 0) atomicOr(io.abort_flag, 1u);
      break;  // block-uniform; the abort flag releases any waiting block
    }
    if (task.kind == kTaskScan) {
      scan_tile_task<TS32, kThreads, kChunks>(seg, task.tile, io, sm.scan.tile, sm.scan.sh, &bar, phase,
                                     [&] { take_next(); });
    } else if (task.kind == kTaskGather) {
      take_next();
      gather_tile_task(seg, task.tile, io);
    } else if (task.kind == kTaskHist) {
      hist_tile_task(seg, task.tile, io, sm.hist.cnt);
      __threadfence();
      __syncthreads();
      if (t == 0) {
        const uint32_t prev = atomicAdd(&ctrl[task.seg].hist_done, 1u);
        s_flag = (prev + 1 == static_cast<uint32_t>(seg.tiles)) ? 1 : 0;
      }
      __syncthreads();
      if (s_flag) {  // last HIST tile of the segment: scan the histogram
        __threadfence();
        block_exclusive_scan_inplace(reinterpret_cast<int32_t *>(io.state + seg.state),
                                     static_cast<int64_t>(seg.buckets) * seg.tiles, sm.hist.wsum);
        __threadfence();
        __syncthreads();
        if (t == 0) st_release_u32(&ctrl[task.seg].ready, 1u);
      }
    } else {
      if (t == 0) {
        bool ok = ld_acquire_u32(&ctrl[task.seg].ready) != 0u;
        if (!ok) {
          const uint64_t t0 = globaltimer_ns();
          while (!(ok = ld_acquire_u32(&ctrl[task.seg].ready) != 0u)) {
            if (globaltimer_ns() - t0 > io.timeout_ns || fault_raised(io.abort_flag)) break;
            __nanosleep(100);
          }
        }
        if (!ok) {
          raise_fault(io.fault, EDPP_FAULT_TIMEOUT);
          atomicOr(io.abort_flag, 1u);
        }
        s_flag = ok ? 1 : 0;
        take_next();
      }
      __syncthreads();
      if (s_flag) split_tile_task(seg, task.tile, io, sm, &bar, phase);
    }
    // this task's generic accesses of shared memory before the next task's
    // bulk copies into it; shared memory and s_task reused by the next task
    fence_proxy_async_smem();
    __syncthreads();
  }
}

// ---- KINDS schedule: one launch per tile kind, one block per tile ----
// Stream order separates the kinds, so no task waits on a flag; scan tiles
// wait only on lower tiles of their own segment (lower block indices).

// Scan tiles as the global look-back scan cuts them: 128 threads x 8
// 16-byte chunks (the same 4096 elements), 10 blocks per SM (12 spilled
// 52 bytes and ran 1.5% slower).
constexpr int kScanThreads = 128, kScanChunks = 8;
using TSK = TileScan<int32_t, kScanThreads, kScanChunks>;

__global__ void __launch_bounds__(kScanThreads, 10)
    kind_scan_kernel(const DevSeg *__restrict__ segs, const DevTask *__restrict__ tasks, TaskIO io) {
  __shared__ alignas(128) int32_t tile[kTile];
  __shared__ TSK::Shared sh;
  __shared__ alignas(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const DevTask task = tasks[blockIdx.x];
  DevSeg seg;
  if (!task_in_plan(task, segs, io, seg)) {
    if (threadIdx.x == 0) atomicOr(io.abort_flag, 1u);  // releases waiting tiles
    return;
  }
  uint32_t phase = 0;
  scan_tile_task<TSK, kScanThreads, kScanChunks>(seg, task.tile, io, tile, sh, &bar, phase, [] {});
}

__global__ void __launch_bounds__(kThreads, 8)
    kind_gather_kernel(const DevSeg *__restrict__ segs, const DevTask *__restrict__ tasks,
                       TaskIO io) {
  const DevTask task = tasks[blockIdx.x];
  DevSeg seg;
  if (task_in_plan(task, segs, io, seg)) gather_tile_task(seg, task.tile, io);
}

__global__ void __launch_bounds__(kThreads, 8)
    kind_hist_kernel(const DevSeg *__restrict__ segs, const DevTask *__restrict__ tasks, TaskIO io) {
  __shared__ uint32_t cnt[kMaxB];
  const DevTask task = tasks[blockIdx.x];
  DevSeg seg;
  if (task_in_plan(task, segs, io, seg)) hist_tile_task(seg, task.tile, io, cnt);
}

// One block per split segment: exclusive scan of its histogram in place.
__global__ void __launch_bounds__(kThreads)
    kind_his_scan_kernel(const DevSeg *__restrict__ segs, const int32_t *__restrict__ split_segs,
                         TaskIO io) {
  __shared__ int32_t wsum[32];
  const int i = split_segs[blockIdx.x];
  if (i < 0 || i >= io.num_segs) {
    if (threadIdx.x == 0) raise_fault(io.fault, EDPP_FAULT_PLAN);
    return;
  }
  const DevSeg seg = segs[i];
  if (seg.op != EDPP_BATCH_SPLIT) {
    if (threadIdx.x == 0) raise_fault(io.fault, EDPP_FAULT_PLAN);
    return;
  }
  block_exclusive_scan_inplace(reinterpret_cast<int32_t *>(io.state + seg.state),
                               static_cast<int64_t>(seg.buckets) * seg.tiles, wsum);
}

__global__ void __launch_bounds__(kThreads, 3)
    kind_split_kernel(const DevSeg *__restrict__ segs, const DevTask *__restrict__ tasks,
                      TaskIO io) {
  __shared__ BatchSmem sm;
  __shared__ alignas(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const DevTask task = tasks[blockIdx.x];
  DevSeg seg;
  uint32_t phase = 0;
  if (task_in_plan(task, segs, io, seg)) split_tile_task(seg, task.tile, io, sm, &bar, phase);
}

}  // namespace

// ---- host planner --------------------------------------------------------------
namespace {

constexpr size_t kHdrB = 256;  // ticket (u64) + abort flag (u32)

int build_plan(const edpp_segment *in, int num, const edpp_batch_tuning *tune, BatchPlanImpl &p) {
  p.num_segs = num;
  p.segs.resize(static_cast<size_t>(num));
  std::vector<int> order(static_cast<size_t>(num));
  std::iota(order.begin(), order.end(), 0);
  const int defer = tune ? std::max(0, tune->split_defer_segments) : 1;
  const bool largest_first = tune ? tune->largest_first != 0 : true;
  p.blocks_per_sm = tune && tune->blocks_per_sm > 0 ? tune->blocks_per_sm : 4;
  p.schedule = tune ? tune->schedule : EDPP_BATCH_SCHEDULE_KINDS;
  if (p.schedule != EDPP_BATCH_SCHEDULE_KINDS && p.schedule != EDPP_BATCH_SCHEDULE_QUEUE)
    return EDPP_EINVAL;
  if (largest_first)
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return in[a].length > in[b].length; });
  // state: scan tile words first (zeroed per launch), then split histograms
  size_t scan_state = 0, split_state = 0;
  for (int i = 0; i < num; ++i) {
    const edpp_segment &s = in[i];
    if (s.length < 0 || s.offset < 0) return EDPP_EINVAL;
    if (s.op != EDPP_BATCH_SCAN && s.op != EDPP_BATCH_SPLIT && s.op != EDPP_BATCH_GATHER)
      return EDPP_EINVAL;
    if (s.op == EDPP_BATCH_SPLIT &&
        (s.buckets < 1 || s.buckets > kMaxB || (s.buckets & (s.buckets - 1))))
      return EDPP_EINVAL;
    DevSeg d{};
    d.off = s.offset;
    d.len = s.length;
    d.op = s.op;
    d.tiles = static_cast<int32_t>((static_cast<int64_t>(s.length) + kTile - 1) / kTile);
    d.buckets = s.op == EDPP_BATCH_SPLIT ? s.buckets : 0;
    if (s.op == EDPP_BATCH_SCAN) {
      d.state = static_cast<int64_t>(scan_state);
      scan_state += LookbackState<int32_t>::bytes(d.tiles);
    }
    p.segs[static_cast<size_t>(i)] = d;
    p.total_elems += s.length;
  }
  for (int i = 0; i < num; ++i) {
    DevSeg &d = p.segs[static_cast<size_t>(i)];
    if (d.op == EDPP_BATCH_SPLIT) {
      d.state = static_cast<int64_t>(scan_state + split_state);
      split_state += round_up(static_cast<size_t>(d.buckets) * d.tiles * 4, 256);
    }
  }
  p.scan_state_bytes = scan_state;
  p.state_bytes = scan_state + split_state;
  // task queue: segments in order; a split's SPLIT tasks follow `defer`
  // segments after its HIST tasks (so the histogram scan overlaps other work)
  std::vector<std::vector<DevTask>> pending;  // deferred split scatter lists
  std::vector<int> pending_age;
  auto flush_due = [&](bool all) {
    for (size_t k = 0; k < pending.size();) {
      if (all || pending_age[k] >= defer) {
        p.tasks.insert(p.tasks.end(), pending[k].begin(), pending[k].end());
        pending.erase(pending.begin() + static_cast<long>(k));
        pending_age.erase(pending_age.begin() + static_cast<long>(k));
      } else {
        ++k;
      }
    }
  };
  for (int oi = 0; oi < num; ++oi) {
    const int i = order[static_cast<size_t>(oi)];
    const DevSeg &d = p.segs[static_cast<size_t>(i)];
    for (auto &a : pending_age) ++a;
    flush_due(false);
    if (d.len == 0) continue;
    if (d.op == EDPP_BATCH_SCAN) {
      for (int t = 0; t < d.tiles; ++t) p.tasks.push_back({i, t, kTaskScan, 0});
    } else if (d.op == EDPP_BATCH_GATHER) {
      for (int t = 0; t < d.tiles; ++t) p.tasks.push_back({i, t, kTaskGather, 0});
    } else {
      for (int t = 0; t < d.tiles; ++t) p.tasks.push_back({i, t, kTaskHist, 0});
      std::vector<DevTask> sc;
      for (int t = 0; t < d.tiles; ++t) sc.push_back({i, t, kTaskSplit, 0});
      pending.push_back(std::move(sc));
      pending_age.push_back(0);
    }
  }
  flush_due(true);
  p.queue_tasks = static_cast<int64_t>(p.tasks.size());
  if (p.schedule == EDPP_BATCH_SCHEDULE_KINDS) {
    // per kind, segments in the given order, tiles ascending
    std::vector<DevTask> scan, gather, split;
    for (int i = 0; i < num; ++i) {
      const DevSeg &d = p.segs[static_cast<size_t>(i)];
      if (d.len == 0) continue;
      auto &dst = d.op == EDPP_BATCH_SCAN ? scan : d.op == EDPP_BATCH_GATHER ? gather : split;
      const int32_t kind = d.op == EDPP_BATCH_SCAN     ? kTaskScan
                           : d.op == EDPP_BATCH_GATHER ? kTaskGather
                                                       : kTaskSplit;
      for (int t = 0; t < d.tiles; ++t) dst.push_back({i, t, kind, 0});
      if (d.op == EDPP_BATCH_SPLIT) p.split_segs.push_back(i);
    }
    p.n_scan = static_cast<int64_t>(scan.size());
    p.n_gather = static_cast<int64_t>(gather.size());
    p.n_split = static_cast<int64_t>(split.size());
    p.tasks = std::move(scan);
    p.tasks.insert(p.tasks.end(), gather.begin(), gather.end());
    p.tasks.insert(p.tasks.end(), split.begin(), split.end());
  }
  // the same layout for both schedules: the task area fits the queue form
  size_t o = kHdrB;
  p.off_segs = o;
  o += round_up(sizeof(DevSeg) * p.segs.size(), 256);
  p.off_tasks = o;
  o += round_up(sizeof(DevTask) * static_cast<size_t>(p.queue_tasks), 256);
  p.off_split_segs = o;
  o += round_up(sizeof(int32_t) * p.segs.size(), 256);
  p.off_ctrl = o;
  o += round_up(sizeof(Ctrl) * p.segs.size(), 256);
  p.off_state = o;
  o += round_up(p.state_bytes, 256);
  p.bytes = o;
  return EDPP_OK;
}

}  // namespace
}  // namespace edpp

using edpp::BatchPlanImpl;

extern "C" {

int edpp_batch_plan_create(const edpp_segment *segs, int num_segs, const edpp_batch_tuning *tuning,
                           edpp_batch_plan **out) {
  if (!out || num_segs < 0 || (num_segs > 0 && !segs)) return EDPP_EINVAL;
  auto *p = new (std::nothrow) edpp_batch_plan;
  if (!p) return EDPP_ENOMEM;
  const int s = edpp::build_plan(segs, num_segs, tuning, p->impl);
  if (s != EDPP_OK) {
    delete p;
    return s;
  }
  *out = p;
  return EDPP_OK;
}

void edpp_batch_plan_destroy(edpp_batch_plan *plan) { delete plan; }

size_t edpp_batch_plan_workspace_size(const edpp_batch_plan *plan) {
  return plan ? plan->impl.bytes : 0;
}

int edpp_batch_plan_num_tasks(const edpp_batch_plan *plan) {
  return plan ? static_cast<int>(plan->impl.queue_tasks) : 0;
}

int edpp_batch_plan_upload(const edpp_batch_plan *plan, void *ws, size_t ws_bytes, void *stream) {
  if (!plan || !ws) return EDPP_EINVAL;
  const BatchPlanImpl &p = plan->impl;
  if (ws_bytes < p.bytes) return EDPP_ENOMEM;
  cudaStream_t st = edpp::as_stream(stream);
  char *w = static_cast<char *>(ws);
  if (!p.segs.empty() &&
      cudaMemcpyAsync(w + p.off_segs, p.segs.data(), sizeof(edpp::DevSeg) * p.segs.size(),
                      cudaMemcpyHostToDevice, st) != cudaSuccess)
    return EDPP_ECUDA;
  if (!p.tasks.empty() &&
      cudaMemcpyAsync(w + p.off_tasks, p.tasks.data(), sizeof(edpp::DevTask) * p.tasks.size(),
                      cudaMemcpyHostToDevice, st) != cudaSuccess)
    return EDPP_ECUDA;
  if (!p.split_segs.empty() &&
      cudaMemcpyAsync(w + p.off_split_segs, p.split_segs.data(),
                      sizeof(int32_t) * p.split_segs.size(), cudaMemcpyHostToDevice,
                      st) != cudaSuccess)
    return EDPP_ECUDA;
  // pageable sources: make the copies complete before the plan can change
  return edpp::cuda_status(cudaStreamSynchronize(st));
}

int edpp_batch_launch(const edpp_batch_plan *plan, const int32_t *in0, const int32_t *in1,
                      int32_t *out0, int32_t *out1, void *ws, size_t ws_bytes, void *stream) {
  using namespace edpp;
  if (!plan || !ws) return EDPP_EINVAL;
  const BatchPlanImpl &p = plan->impl;
  if (ws_bytes < p.bytes) return EDPP_ENOMEM;
  if (p.tasks.empty()) return EDPP_OK;
  if (!in0 || !out0) return EDPP_EINVAL;
  // gather tiles read in1 (indices); split tiles read in1 and write out1 (values)
  if ((p.n_gather || p.n_split) && !in1) return EDPP_EINVAL;
  if (p.n_split && !out1) return EDPP_EINVAL;
  unsigned *fault = fault_word();
  if (!fault) return EDPP_ECUDA;
  cudaStream_t st = as_stream(stream);
  char *w = static_cast<char *>(ws);
  // zero: ticket + abort flag, per-segment control words, scan tile states
  if (cudaMemsetAsync(w, 0, kHdrB, st) != cudaSuccess) return EDPP_ECUDA;
  if (cudaMemsetAsync(w + p.off_ctrl, 0, p.off_state - p.off_ctrl + p.scan_state_bytes, st) !=
      cudaSuccess)
    return EDPP_ECUDA;
  const DevSeg *dsegs = reinterpret_cast<const DevSeg *>(w + p.off_segs);
  const DevTask *dtasks = reinterpret_cast<const DevTask *>(w + p.off_tasks);
  const TaskIO io{in0, in1, out0, out1, w + p.off_state, kDefaultWaitNs, fault,
                  reinterpret_cast<unsigned *>(w + 8), aligned16(in0), aligned16(in1),
                  p.num_segs};
  if (p.schedule == EDPP_BATCH_SCHEDULE_KINDS) {
    if (p.n_scan)
      kind_scan_kernel<<<static_cast<unsigned>(p.n_scan), kScanThreads, 0, st>>>(dsegs, dtasks,
                                                                                 io);
    if (p.n_gather)
      kind_gather_kernel<<<static_cast<unsigned>(p.n_gather), kThreads, 0, st>>>(
          dsegs, dtasks + p.n_scan, io);
    if (p.n_split) {
      const DevTask *split_tasks = dtasks + p.n_scan + p.n_gather;
      kind_hist_kernel<<<static_cast<unsigned>(p.n_split), kThreads, 0, st>>>(dsegs, split_tasks,
                                                                              io);
      kind_his_scan_kernel<<<static_cast<unsigned>(p.split_segs.size()), kThreads, 0, st>>>(
          dsegs, reinterpret_cast<const int32_t *>(w + p.off_split_segs), io);
      kind_split_kernel<<<static_cast<unsigned>(p.n_split), kThreads, 0, st>>>(dsegs, split_tasks,
                                                                               io);
    }
    return launch_status();
  }
  static std::once_flag occ_once[64];
  static cudaError_t occ_err[64];
  static int resident[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::call_once(occ_once[dev], [dev] {
    occ_err[dev] = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident[dev], batch_kernel,
                                                                 kThreads, 0);
  });
  if (occ_err[dev] != cudaSuccess) return EDPP_ECUDA;
  // blocks beyond what stays resident would only start once the queue is empty
  const int per_sm = std::max(1, std::min(p.blocks_per_sm, resident[dev]));
  int64_t blocks = static_cast<int64_t>(device_sm_count()) * per_sm;
  blocks = min64(blocks, static_cast<int64_t>(p.tasks.size()));
  batch_kernel<<<static_cast<unsigned>(max64(blocks, 1)), kThreads, 0, st>>>(
      dsegs, dtasks, static_cast<int>(p.tasks.size()), io,
      reinterpret_cast<Ctrl *>(w + p.off_ctrl), reinterpret_cast<unsigned long long *>(w));
  return launch_status();
}

}  // extern "C"

// ---- plain per-array launches (the baseline the batch replaces) ---------------
namespace {
constexpr int kNeedIn0Out0 = 1, kNeedIn1 = 2, kNeedOut1 = 4;
// Which of the caller's arrays the segments touch: every non-empty segment
// reads in0 and writes out0; gathers read in1 (indices); splits read in1
// and write out1 (values).
int batch_io_needs(const edpp_segment *segs, int num_segs) {
  int need = 0;
  for (int i = 0; i < num_segs; ++i) {
    if (segs[i].length <= 0) continue;
    need |= kNeedIn0Out0;
    if (segs[i].op == EDPP_BATCH_GATHER) need |= kNeedIn1;
    if (segs[i].op == EDPP_BATCH_SPLIT) need |= kNeedIn1 | kNeedOut1;
  }
  return need;
}
}  // namespace

extern "C" size_t edpp_batch_plain_workspace_size(const edpp_segment *segs, int num_segs) {
  size_t m = 0;
  for (int i = 0; i < num_segs; ++i) {
    const edpp_segment &s = segs[i];
    size_t b = 0;
    if (s.op == EDPP_BATCH_SCAN) b = edpp_scan_workspace_size(s.length, EDPP_I32, EDPP_SCAN_LOOKBACK);
    else if (s.op == EDPP_BATCH_SPLIT) b = edpp_split_workspace_size(s.length, s.buckets, EDPP_KVS_SOA);
    m = std::max(m, b);
  }
  return m;
}

// One C-ABI call per segment, issued back to back on `stream` from this host
// loop; one workspace serves every call (calls are ordered on the stream).
// Gather segments use segment-local indices, so they run as one-pass gathers
// of the segment's slice.
extern "C" int edpp_batch_run_plain(const edpp_segment *segs, int num_segs, const int32_t *in0,
                                    const int32_t *in1, int32_t *out0, int32_t *out1, void *ws,
                                    size_t ws_bytes, void *stream) {
  if (num_segs > 0 && !segs) return EDPP_EINVAL;
  const int need = batch_io_needs(segs, num_segs);
  if ((need & kNeedIn0Out0) && (!in0 || !out0)) return EDPP_EINVAL;
  if ((need & kNeedIn1) && !in1) return EDPP_EINVAL;
  if ((need & kNeedOut1) && !out1) return EDPP_EINVAL;
  for (int i = 0; i < num_segs; ++i) {
    const edpp_segment &s = segs[i];
    if (s.length == 0) continue;
    int st;
    if (s.op == EDPP_BATCH_SCAN)
      st = edpp_scan_exclusive_i32(in0 + s.offset, out0 + s.offset, s.length, EDPP_SCAN_LOOKBACK,
                                   ws, ws_bytes, stream);
    else if (s.op == EDPP_BATCH_SPLIT)
      st = edpp_split_i32(in0 + s.offset, out0 + s.offset, nullptr, s.length, s.buckets,
                          EDPP_KVS_SOA, in1 + s.offset, out1 + s.offset, ws, ws_bytes, stream);
    else if (s.op == EDPP_BATCH_GATHER)
      st = edpp_gather_i32(in0 + s.offset, out0 + s.offset, s.length, in1 + s.offset, 1, stream);
    else
      st = EDPP_EINVAL;
    if (st != EDPP_OK) return st;
  }
  return EDPP_OK;
}

// ---- autotuner ----------------------------------------------------------------------
// Times every candidate schedule on this GPU for the given segments (CUDA
// events around `reps` launches after one warm-up) and returns the fastest.
// Candidates: the KINDS schedule, and the QUEUE schedule with blocks per SM
// {1,2,3,4} x split deferral {0,1,2,4} x segment order {given, largest
// first}.  The workspace must fit the plan (edpp_batch_plan_workspace_size;
// it does not depend on the tuning).
extern "C" int edpp_batch_autotune(const edpp_segment *segs, int num_segs, const int32_t *in0,
                                   const int32_t *in1, int32_t *out0, int32_t *out1, void *ws,
                                   size_t ws_bytes, void *stream, int reps,
                                   edpp_batch_tuning *best, float *best_ms) {
  if (!best || reps < 1) return EDPP_EINVAL;
  if (num_segs > 0 && !segs) return EDPP_EINVAL;
  const int need = batch_io_needs(segs, num_segs);
  if ((need & kNeedIn0Out0) && (!in0 || !out0)) return EDPP_EINVAL;
  if ((need & kNeedIn1) && !in1) return EDPP_EINVAL;
  if ((need & kNeedOut1) && !out1) return EDPP_EINVAL;
  cudaStream_t st = edpp::as_stream(stream);
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess) return EDPP_ECUDA;
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(a);
    return EDPP_ECUDA;
  }
  float best_t = 1e30f;
  int status = EDPP_OK;
  std::vector<edpp_batch_tuning> cands{{0, 0, 0, EDPP_BATCH_SCHEDULE_KINDS}};
  for (int bps : {1, 2, 3, 4})  // the launch clamps to the resident count
    for (int defer : {0, 1, 2, 4})
      for (int lf : {0, 1}) cands.push_back({bps, defer, lf, EDPP_BATCH_SCHEDULE_QUEUE});
  for (const edpp_batch_tuning &tu : cands) {
    edpp_batch_plan *plan = nullptr;
    status = edpp_batch_plan_create(segs, num_segs, &tu, &plan);
    if (status != EDPP_OK) break;
    status = edpp_batch_plan_upload(plan, ws, ws_bytes, stream);
    if (status == EDPP_OK)
      status = edpp_batch_launch(plan, in0, in1, out0, out1, ws, ws_bytes, stream);
    if (status == EDPP_OK && cudaEventRecord(a, st) != cudaSuccess) status = EDPP_ECUDA;
    for (int r = 0; r < reps && status == EDPP_OK; ++r)
      status = edpp_batch_launch(plan, in0, in1, out0, out1, ws, ws_bytes, stream);
    if (status == EDPP_OK && cudaEventRecord(b, st) != cudaSuccess) status = EDPP_ECUDA;
    if (status == EDPP_OK) status = edpp_sync_status(stream, 0);
    float ms = 0;
    if (status == EDPP_OK && cudaEventElapsedTime(&ms, a, b) != cudaSuccess) status = EDPP_ECUDA;
    edpp_batch_plan_destroy(plan);
    if (status != EDPP_OK) break;
    ms /= reps;
    if (ms < best_t) {
      best_t = ms;
      *best = tu;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (best_ms) *best_ms = best_t;
  return status;
}
