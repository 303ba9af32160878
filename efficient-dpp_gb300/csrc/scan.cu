// scan.cu — global exclusive / inclusive prefix sums of int32, int64, f32.
//
// Three schemes, all producing the same integer results:
//
//  LOOKBACK  one launch, one tile per block, tiles taken from an atomic
//            ticket so progress never depends on launch order; a tile's
//            exclusive prefix comes from a decoupled look-back over the
//            published aggregates of its predecessors (bounded waits).
//            Traffic 2n: each element read once and written once.  Stands
//            in for the reference's chained scan with adjacent
//            synchronisation (opencl/primitives/scanImpl.cpp:15-66,
//            opencl/kernels/scan_global_chain_kernel.cl:11-203), whose
//            tile t waits for tile t-1 only and spins without a limit.
//  RTS       reduce-then-scan in three launches (per-block reduction, scan of
//            the block sums in one block, per-block rescan with the offset):
//            traffic 3n.  The reference's RSS scan
//            (opencl/primitives/scanImpl.cpp:69-160,
//            opencl/kernels/scan_global_RSS_kernel.cl:142-240) and
//            scan_RTS_omp (openmp/test_scan_CPU.cpp:125-163).
//  SSA       scan-then-propagate ("scan-scan-add"): per-block scans written
//            out, scan of block sums, then an add pass: traffic 4n.
//            scan_SSA_omp (openmp/test_scan_CPU.cpp:85-122).
//
// Tiles are staged into shared memory by one 1-D TMA bulk copy
// (cp.async.bulk) when the input is 16-byte aligned; see scan_tile.cuh for
// the tile layout.
#include <algorithm>
#include <mutex>

#include "scan_tile.cuh"
#include "tune.h"

namespace edpp {
namespace {

constexpr int kThreads = 256;
constexpr int kChunks = 4;  // 16-byte chunks per thread: 16 KB tiles

// Workspace header: [0] tile ticket counter (u64), [8] the call's abort flag
// (u32).  Zeroed with the look-back state before every call.
constexpr size_t kHeader = 256;
// Upper bound on blocks of the RTS / SSA schemes (per-block partial sums).
constexpr int64_t kMaxChunkBlocks = 8192;

template <typename T> using TS = TileScan<T, kThreads, kChunks>;
// Look-back tile shapes (threads per block, 16-byte chunks per thread, blocks
// per SM for 4- / 8-byte elements), chosen per size class by the tuning
// table (edpp_tune_*):
//   variant 0  128 x 8   16 KB tiles, 12 / 8 blocks per SM (the default:
//              fewer warps idle at the barrier while warp 0 looks back)
//   variant 1  256 x 8   32 KB tiles,  6 / 4 blocks per SM (half the tiles,
//              so half the look-backs)
//   variant 2  512 x 4   32 KB tiles,  6 / 4 blocks per SM
//   variant 3  512 x 8   64 KB tiles,  3 / 2 blocks per SM (a quarter of the
//              look-backs)
// Variant 0's tiles are the smallest; tile state and workspace are sized
// for them, so every shape fits the same workspace.
constexpr int kLbThreads = 128;
constexpr int kLbChunks = 8;
constexpr int kLbVariants = 4;
template <typename T> using TSL = TileScan<T, kLbThreads, kLbChunks>;
static_assert(TSL<int32_t>::kTile == TS<int32_t>::kTile && TSL<int64_t>::kTile == TS<int64_t>::kTile,
              "look-back tiles match the other schemes' tiles");

// ---- LOOKBACK ----------------------------------------------------------------
// Tile = block index (+ tile_base).  Blocks of a 1-D grid are dispatched
// in index order, so every predecessor of a running tile has been dispatched
// and keeps running: the look-back waits end (they are bounded regardless).
// Measured at 2^30 int32 against an atomic tile ticket and 8 blocks of 256
// threads: block-index tiles 13% faster, then 12 blocks of 128 threads per
// SM another 12%.
template <typename T, bool kInclusive, int TH = kLbThreads, int CH = kLbChunks,
          int MINB = (sizeof(T) == 4 ? 12 : 8)>
__global__ void __launch_bounds__(TH, MINB)
    scan_lookback_kernel(const T *in, T *out, int64_t n, int64_t num_tiles,
                         unsigned long long *ticket, LookbackState<T> st, int64_t tile_base,
                         bool tma, bool vec_out, uint64_t timeout_ns, unsigned *fault) {
  using S = TileScan<T, TH, CH>;
  constexpr int kTile = S::kTile;
  __shared__ alignas(128) T tile[kTile];
  __shared__ typename S::Shared sh;
  __shared__ alignas(8) uint64_t bar;
  __shared__ int64_t s_tile;

  unsigned *abort_flag = reinterpret_cast<unsigned *>(ticket + 1);
  if (threadIdx.x == 0) {
    s_tile = static_cast<int64_t>(blockIdx.x) + tile_base;
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int64_t t = s_tile;
  if (t >= num_tiles) return;
  const int64_t base = t * kTile;
  const int count = static_cast<int>(min64(kTile, n - base));

  const uint32_t bulk = stage_tile<T, kTile, TH>(tile, in + base, count, tma, &bar);
  if (bulk) {
    if (!mbar_wait_bounded(&bar, 0, timeout_ns, fault)) return;
  }
  if (count < kTile || !bulk) __syncthreads();

  Chunk<T> c[CH];
  T wex[CH];
  S::phase1(tile, c, wex, sh);
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const T agg = S::phase2_warp0(sh, lane);
    T prefix = zero_of<T>();
    bool ok = true;
    if (t == 0) {
      if (lane == 0) st.publish(0, kFlagIncl, agg);
    } else {
      prefix = lookback_warp<T>(st, t, agg, lane, timeout_ns, fault, abort_flag, ok);
    }
    if (lane == 0) sh.prefix = ok ? prefix : zero_of<T>();
  }
  __syncthreads();
  if (fault_raised(abort_flag)) return;  // a failed call writes nothing further
  S::template phase3<kInclusive>(c, wex, sh, sh.prefix);
  S::store(out, base, count, c, vec_out);
}

// ---- RTS / SSA building blocks ----------------------------------------------

// Sum of in[lo, hi) by the whole block; the result is valid in thread 0.
// lo is a multiple of the tile size (16-byte aligned when vec).  kKeep: the
// range is read again soon (the fused RTS), so its lines are loaded with the
// normal L2 policy instead of evict-first.
template <typename T, bool kKeep = false>
__device__ __forceinline__ T block_reduce_range(const T *in, int64_t lo, int64_t hi, bool vec) {
  T acc = zero_of<T>();
  if (lo < hi) {
    constexpr int E = Chunk<T>::E;
    if (vec) {  // lo is a multiple of the tile size, hence 16-byte aligned
      const int64_t nv = (hi - lo) / E;
      const uint4 *p = reinterpret_cast<const uint4 *>(in + lo);
      int64_t i = threadIdx.x;
      for (; i + 3 * kThreads < nv; i += 4 * kThreads) {
        Chunk<T> c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) c[u].raw = kKeep ? __ldcg(p + i + u * kThreads) : __ldcs(p + i + u * kThreads);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int e = 0; e < E; ++e) acc = op_add(acc, c[u].e[e]);
      }
      for (; i < nv; i += kThreads) {
        Chunk<T> c;
        c.raw = kKeep ? __ldcg(p + i) : __ldcs(p + i);
#pragma unroll
        for (int e = 0; e < E; ++e) acc = op_add(acc, c.e[e]);
      }
      for (int64_t j = lo + nv * E + threadIdx.x; j < hi; j += kThreads) acc = op_add(acc, in[j]);
    } else {
      for (int64_t j = lo + threadIdx.x; j < hi; j += kThreads) acc = op_add(acc, in[j]);
    }
  }
  __shared__ T ws[kThreads / 32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
  __syncthreads();
  T v = zero_of<T>();
  if (threadIdx.x < 32) {
    v = threadIdx.x < kThreads / 32 ? ws[threadIdx.x] : zero_of<T>();
    v = warp_sum(v);
  }
  return v;
}

// Per-block sum of the block's contiguous range [b*per, min((b+1)*per, n)).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    reduce_blocks_kernel(const T *in, int64_t n, int64_t per, T *partials, bool vec) {
  const int64_t lo = static_cast<int64_t>(blockIdx.x) * per;
  const int64_t hi = min64(n, lo + per);
  const T v = block_reduce_range(in, lo, hi, vec);
  if (threadIdx.x == 0) partials[blockIdx.x] = v;
}

// Exclusive scan of `m` partial sums in place, one block of 1024 threads.
template <typename T> __global__ void __launch_bounds__(1024) scan_partials_kernel(T *p, int m) {
  __shared__ T wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (m + 1023) / 1024;
  const int lo = min(m, t * per), hi = min(m, lo + per);
  T s = zero_of<T>();
  for (int i = lo; i < hi; ++i) s = op_add(s, p[i]);
  const T si = warp_incl_scan(s, lane);
  if (lane == 31) wsum[w] = si;
  __syncthreads();
  if (w == 0) {
    const T x = wsum[lane];
    const T xi = warp_incl_scan(x, lane);
    const T ex = shfl_up(xi, 1);
    wsum[lane] = lane == 0 ? zero_of<T>() : ex;
  }
  __syncthreads();
  const T ex_t = shfl_up(si, 1);
  T run = op_add(wsum[w], lane == 0 ? zero_of<T>() : ex_t);
  for (int i = lo; i < hi; ++i) {
    const T v = p[i];
    p[i] = run;
    run = op_add(run, v);
  }
}

// Block b scans its tiles [b*tpb, (b+1)*tpb) in order, starting from offset
// `offsets[b]` (RTS) or 0 (SSA, which then records its block total in
// totals[b]).  Tiles are double-buffered: the bulk copy of tile i+1 is in
// flight while tile i is scanned.
// Scan tiles [t_lo, t_hi) in order starting from `running`; returns the
// running sum after the last tile (false: a bulk copy timed out).  `bar`
// must be initialised; buffers and barriers are the caller's shared memory.
// `phase` (bit s: parity of bar[s]'s next completion) carries over between
// calls on the same barriers.
template <typename T, bool kInclusive, bool kStreamOut = false, bool kLastUse = false>
__device__ bool scan_tile_run(const T *in, T *out, int64_t n, int64_t t_lo, int64_t t_hi,
                              T &running, T (*buf)[TS<T>::kTile], typename TS<T>::Shared &sh,
                              uint64_t *bar, uint32_t &phase, bool tma, bool vec_out,
                              uint64_t timeout_ns, unsigned *fault) {
  using S = TS<T>;
  constexpr int kTile = S::kTile;
  auto count_of = [&](int64_t t) { return static_cast<int>(min64(kTile, n - t * kTile)); };
  // Prologue: stage the first tile.
  const uint64_t policy = kLastUse ? l2_policy_evict_first() : 0;
  uint32_t bulk_cur = stage_tile<T, kTile, kThreads, kLastUse>(buf[0], in + t_lo * kTile,
                                                               count_of(t_lo), tma, &bar[0], policy);
  for (int64_t t = t_lo; t < t_hi; ++t) {
    const int slot = static_cast<int>((t - t_lo) & 1);
    const int count = count_of(t);
    // Prefetch the next tile into the other buffer (free since the last
    // barrier of the previous iteration).
    uint32_t bulk_next = 0;
    if (t + 1 < t_hi)
      bulk_next = stage_tile<T, kTile, kThreads, kLastUse>(buf[slot ^ 1], in + (t + 1) * kTile,
                                                           count_of(t + 1), tma, &bar[slot ^ 1],
                                                           policy);
    if (bulk_cur) {
      if (!mbar_wait_bounded(&bar[slot], (phase >> slot) & 1u, timeout_ns, fault)) return false;
      phase ^= 1u << slot;
    }
    __syncthreads();  // plain-load part of both buffers visible
    Chunk<T> c[kChunks];
    T wex[kChunks];
    S::phase1(buf[slot], c, wex, sh);
    __syncthreads();
    if (threadIdx.x < 32) {
      const T agg = S::phase2_warp0(sh, threadIdx.x);
      if (threadIdx.x == 0) sh.total = agg;
    }
    __syncthreads();
    S::template phase3<kInclusive>(c, wex, sh, running);
    S::template store<kStreamOut>(out, t * kTile, count, c, vec_out);
    running = op_add(running, sh.total);
    bulk_cur = bulk_next;
    __syncthreads();  // everyone done with buf[slot] and sh before reuse
  }
  return true;
}

template <typename T, bool kInclusive, bool kFromOffsets>
__global__ void __launch_bounds__(kThreads)
    scan_blocks_kernel(const T *in, T *out, int64_t n, int64_t tpb, const T *offsets, T *totals,
                       bool tma, bool vec_out, uint64_t timeout_ns, unsigned *fault) {
  using S = TS<T>;
  constexpr int kTile = S::kTile;
  __shared__ alignas(128) T buf[2][kTile];
  __shared__ typename S::Shared sh;
  __shared__ alignas(8) uint64_t bar[2];
  const int64_t num_tiles = (n + kTile - 1) / kTile;
  const int64_t t_lo = static_cast<int64_t>(blockIdx.x) * tpb;
  const int64_t t_hi = min64(num_tiles, t_lo + tpb);
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  T running = kFromOffsets ? offsets[blockIdx.x] : zero_of<T>();
  uint32_t phase = 0;
  if (t_lo < t_hi &&
      !scan_tile_run<T, kInclusive>(in, out, n, t_lo, t_hi, running, buf, sh, bar, phase, tma,
                                    vec_out, timeout_ns, fault))
    return;
  if (!kFromOffsets && threadIdx.x == 0) totals[blockIdx.x] = running;
}

// One-launch reduce-then-scan for inputs that fit in L2: every block reduces
// its run of tiles (the lines stay in L2), the last block to publish its sum
// releases the others (bounded wait), every block adds up the sums of the
// blocks before it, then scans its tiles again from L2, streaming the output.
// Launched cooperatively, so all blocks are resident together.
template <typename T, bool kInclusive>
__global__ void __launch_bounds__(kThreads)
    rts_fused_kernel(const T *in, T *out, int64_t n, int64_t tpb, T *partials, unsigned *ctl,
                     bool tma, bool vec_out, uint64_t timeout_ns, unsigned *fault) {
  using S = TS<T>;
  constexpr int kTile = S::kTile;
  __shared__ alignas(128) T buf[2][kTile];
  __shared__ typename S::Shared sh;
  __shared__ alignas(8) uint64_t bar[2];
  __shared__ int s_last, s_ok;
  const int64_t num_tiles = (n + kTile - 1) / kTile;
  const int64_t t_lo = static_cast<int64_t>(blockIdx.x) * tpb;
  const int64_t t_hi = min64(num_tiles, t_lo + tpb);
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  // 1. block sum of my tiles, their lines kept in L2 for the second read
  const T agg = t_lo < t_hi
                    ? block_reduce_range<T, true>(in, t_lo * kTile, min64(n, t_hi * kTile), tma)
                    : zero_of<T>();
  if (tid == 0) {
    partials[blockIdx.x] = agg;
    __threadfence();
    s_last = atomicAdd(&ctl[0], 1u) + 1u == gridDim.x;
  }
  __syncthreads();
  // 2. the last block to publish its sum releases the others at once
  if (s_last && tid == 0) {
    __threadfence();
    st_release_u32(&ctl[1], 1u);
  }
  // 3. wait for every block sum (bounded)
  if (tid == 0) {
    bool ok = ld_acquire_u32(&ctl[1]) != 0u;
    if (!ok) {
      const uint64_t t0 = globaltimer_ns();
      while (!(ok = ld_acquire_u32(&ctl[1]) != 0u)) {
        if (globaltimer_ns() - t0 > timeout_ns) break;
        __nanosleep(64);
      }
    }
    if (!ok) raise_fault(fault, EDPP_FAULT_TIMEOUT);
    s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  if (!s_ok) return;
  // every block adds up the sums of the blocks before it itself (at most a
  // few thousand values from L2), instead of one block scanning them all
  // while the others wait
  T pre = zero_of<T>();
  for (int i = tid; i < static_cast<int>(blockIdx.x); i += kThreads)
    pre = op_add(pre, __ldcg(partials + i));
  __shared__ T s_pre[kThreads / 32];
  pre = warp_sum(pre);
  if ((tid & 31) == 0) s_pre[tid >> 5] = pre;
  __syncthreads();
  T running = zero_of<T>();
#pragma unroll
  for (int k = 0; k < kThreads / 32; ++k) running = op_add(running, s_pre[k]);
  // 4. scan the tiles again from L2; the output streams out (evict-first),
  // so it does not push the input's remaining lines out of L2
  uint32_t phase = 0;
  if (t_lo < t_hi)
    scan_tile_run<T, kInclusive, true>(in, out, n, t_lo, t_hi, running, buf, sh, bar, phase, tma,
                                       vec_out, timeout_ns, fault);
}

// Reduce-then-scan for inputs larger than L2, in one cooperative launch.  A
// persistent grid of G blocks walks the input in chunks of G slices of
// kSliceTiles tiles; block b owns slice b of every chunk.  In iteration c a
// block first reduces its slice of chunk c+1 (read from DRAM with the normal
// L2 policy, so its lines stay in L2) and publishes the sum, then waits until
// all G sums of chunk c are published (they were, one iteration earlier,
// unless some block lags by a whole iteration), adds up the sums of the
// slices before its own and the chunk total, and scans its slice of chunk c
// again, from L2, streaming the output (evict-first, so it does not push the
// next chunk's lines out).  DRAM traffic is 8 bytes per int32 element, as for
// the look-back scan, with no chain of tile-to-tile waits: the only wait is
// one count per chunk, a whole iteration after it started filling.  Waits are
// bounded; a block that gives up raises EDPP_FAULT_TIMEOUT and sets the
// call's abort flag so the others stop too.
// kSliceTiles is the slice length in tiles, chosen per size class by the
// tuning table: variant 0 two tiles (the default), variant 1 one tile,
// variant 2 four tiles (reduced in two rounds of eight 16-byte loads per
// thread), variant 3 two tiles with L2 eviction hints (kHint: the reduce's
// loads evict-last, the second read's bulk copies evict-first), variant 4
// two tiles also for inputs that fit L2 (instead of the one-launch fused
// form).  The workspace is sized for one-tile slices, the most.
constexpr int kRtsVariants = 5;

template <typename T, bool kInclusive, int kSliceTiles, bool kHint = false>
__global__ void __launch_bounds__(kThreads, 4)
    rts_chunked_kernel(const T *in, T *out, int64_t n, int64_t chunks, T *sums, unsigned *cnt,
                       unsigned *abort_flag, bool tma, bool vec_out, uint64_t timeout_ns,
                       unsigned *fault) {
  using S = TS<T>;
  constexpr int kTile = S::kTile;
  __shared__ alignas(128) T buf[2][kTile];
  __shared__ typename S::Shared sh;
  __shared__ alignas(8) uint64_t bar[2];
  __shared__ T s_red[2][kThreads / 32];
  __shared__ int s_ok;
  const int64_t G = gridDim.x, b = blockIdx.x;
  const int64_t num_tiles = (n + kTile - 1) / kTile;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  const uint64_t keep = kHint ? l2_policy_evict_last() : 0;
  auto reduce_publish = [&](int64_t c) {
    const int64_t lo = min64(n, (c * G + b) * kSliceTiles * kTile);
    const int64_t hi = min64(n, lo + kSliceTiles * kTile);
    T v;
    if (tma && hi - lo == kSliceTiles * kTile) {
      // a whole slice: up to eight 16-byte loads per thread in flight at once
      constexpr int kV = kSliceTiles * kChunks;
      constexpr int kRound = kV < 8 ? kV : 8;
      constexpr int E = Chunk<T>::E;
      const uint4 *p = reinterpret_cast<const uint4 *>(in + lo);
      T acc = zero_of<T>();
#pragma unroll
      for (int r0 = 0; r0 < kV; r0 += kRound) {
        Chunk<T> q[kRound];
#pragma unroll
        for (int k = 0; k < kRound; ++k)
          q[k].raw = kHint ? ld_v4_policy(p + (r0 + k) * kThreads + tid, keep)
                           : __ldcg(p + (r0 + k) * kThreads + tid);
#pragma unroll
        for (int k = 0; k < kRound; ++k)
#pragma unroll
          for (int e = 0; e < E; ++e) acc = op_add(acc, q[k].e[e]);
      }
      acc = warp_sum(acc);
      if ((tid & 31) == 0) s_red[0][tid >> 5] = acc;
      __syncthreads();
      v = zero_of<T>();
      if (tid == 0) {
#pragma unroll
        for (int k = 0; k < kThreads / 32; ++k) v = op_add(v, s_red[0][k]);
      }
      __syncthreads();  // s_red is reused below
    } else {
      v = block_reduce_range<T, true>(in, lo, hi, tma);  // valid in thread 0
    }
    if (tid == 0) {
      sums[c * G + b] = v;
      __threadfence();  // the sum is visible before the count that announces it
      atomicAdd(&cnt[c], 1u);
    }
  };
  reduce_publish(0);
  T base = zero_of<T>();
  uint32_t phase = 0;
  for (int64_t c = 0; c < chunks; ++c) {
    if (c + 1 < chunks) reduce_publish(c + 1);
    if (tid == 0) {
      const uint32_t need = static_cast<uint32_t>(G);
      bool ok = ld_acquire_u32(&cnt[c]) >= need;
      if (!ok) {
        const uint64_t t0 = globaltimer_ns();
        while (!(ok = ld_acquire_u32(&cnt[c]) >= need)) {
          if (globaltimer_ns() - t0 > timeout_ns || fault_raised(abort_flag)) break;
          __nanosleep(128);
        }
      }
      if (!ok) {
        raise_fault(fault, EDPP_FAULT_TIMEOUT);
        atomicOr(abort_flag, 1u);
      }
      s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    if (!s_ok) return;
    // sums of the slices before this block's, and the chunk total
    T pre = zero_of<T>(), tot = zero_of<T>();
    for (int64_t i = tid; i < G; i += kThreads) {
      const T v = __ldcg(sums + c * G + i);
      tot = op_add(tot, v);
      if (i < b) pre = op_add(pre, v);
    }
    pre = warp_sum(pre);
    tot = warp_sum(tot);
    if ((tid & 31) == 0) {
      s_red[0][tid >> 5] = pre;
      s_red[1][tid >> 5] = tot;
    }
    __syncthreads();
    pre = zero_of<T>();
    tot = zero_of<T>();
#pragma unroll
    for (int k = 0; k < kThreads / 32; ++k) {
      pre = op_add(pre, s_red[0][k]);
      tot = op_add(tot, s_red[1][k]);
    }
    const int64_t t_lo = (c * G + b) * kSliceTiles;
    const int64_t t_hi = min64(num_tiles, t_lo + kSliceTiles);
    T running = op_add(base, pre);
    if (t_lo < t_hi &&
        !scan_tile_run<T, kInclusive, true, kHint>(in, out, n, t_lo, t_hi, running, buf, sh, bar,
                                                   phase, tma, vec_out, timeout_ns, fault))
      return;
    base = op_add(base, tot);
    __syncthreads();  // s_red is rewritten in the next iteration
  }
}

// SSA third pass: out[range of block b] += offsets[b].
template <typename T>
__global__ void __launch_bounds__(kThreads)
    add_offsets_kernel(T *out, int64_t n, int64_t per, const T *offsets, bool vec) {
  const int64_t lo = static_cast<int64_t>(blockIdx.x) * per;
  const int64_t hi = min64(n, lo + per);
  if (lo >= hi) return;
  const T off = offsets[blockIdx.x];
  constexpr int E = Chunk<T>::E;
  if (vec) {
    const int64_t nv = (hi - lo) / E;
    uint4 *p = reinterpret_cast<uint4 *>(out + lo);
    int64_t i = threadIdx.x;
    for (; i + 3 * kThreads < nv; i += 4 * kThreads) {
      Chunk<T> c[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) c[u].raw = p[i + u * kThreads];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
#pragma unroll
        for (int e = 0; e < E; ++e) c[u].e[e] = op_add(off, c[u].e[e]);
        p[i + u * kThreads] = c[u].raw;
      }
    }
    for (; i < nv; i += kThreads) {
      Chunk<T> c;
      c.raw = p[i];
#pragma unroll
      for (int e = 0; e < E; ++e) c.e[e] = op_add(off, c.e[e]);
      p[i] = c.raw;
    }
    for (int64_t j = lo + nv * E + threadIdx.x; j < hi; j += kThreads) out[j] = op_add(off, out[j]);
  } else {
    for (int64_t j = lo + threadIdx.x; j < hi; j += kThreads) out[j] = op_add(off, out[j]);
  }
}

// ---- host side ----------------------------------------------------------------

template <typename T> int64_t tiles_of(int64_t n) {
  return (n + TS<T>::kTile - 1) / TS<T>::kTile;
}

// The chunked RTS: chunks * G slice sums (chunks * G <= slices + G) and one
// count per chunk (chunks <= slices), after the header; sized for the
// shortest slices (one tile).
template <typename T> int64_t slices_of(int64_t n, int slice_tiles = 1) {
  return (tiles_of<T>(n) + slice_tiles - 1) / slice_tiles;
}
template <typename T> size_t chunked_sums_bytes(int64_t n) {
  return round_up(static_cast<size_t>(slices_of<T>(n) + kMaxChunkBlocks) * sizeof(T), 256);
}

template <typename T> size_t workspace_bytes(int64_t n, int algo) {
  if (n <= 0) return 0;
  if (algo == EDPP_SCAN_LOOKBACK) return kHeader + LookbackState<T>::bytes(tiles_of<T>(n));
  const size_t three = kHeader + round_up(static_cast<size_t>(kMaxChunkBlocks) * sizeof(T), 256);
  if (algo != EDPP_SCAN_RTS) return three;
  const size_t chunked = kHeader + chunked_sums_bytes<T>(n) +
                         round_up(static_cast<size_t>(slices_of<T>(n)) * 4, 256);
  return std::max(three, chunked);
}

// Blocks of the RTS / SSA schemes: a few waves of resident blocks, each
// owning a contiguous run of whole tiles.
template <typename T> void chunk_grid(int64_t n, int64_t &blocks, int64_t &tpb) {
  const int64_t tiles = tiles_of<T>(n);
  int64_t g = static_cast<int64_t>(device_sm_count()) * 4;
  g = std::min<int64_t>(g, kMaxChunkBlocks);
  g = std::min<int64_t>(g, tiles);
  tpb = (tiles + g - 1) / g;
  blocks = (tiles + tpb - 1) / tpb;
}

// One look-back launch with tile shape TH x CH (MINB4 / MINB8 blocks per SM
// for 4- / 8-byte elements).  Zeroes the header and the state it uses.
template <typename T, bool kInclusive, int TH, int CH, int MINB4, int MINB8>
int launch_lookback(const T *in, T *out, int64_t n, char *w, cudaStream_t st, int64_t tile_base,
                    bool tma, bool vec_out, uint64_t timeout_ns, unsigned *fault) {
  constexpr int64_t kTileS = TileScan<T, TH, CH>::kTile;
  const int64_t tiles = (n + kTileS - 1) / kTileS;
  if (cudaMemsetAsync(w, 0, kHeader + LookbackState<T>::bytes(tiles), st) != cudaSuccess)
    return EDPP_ECUDA;
  LookbackState<T> state;
  state.bind(w + kHeader, tiles);
  // One block per tile, in block-index order.  (A persistent form that
  // prefetches its next tile measured 10-15% slower: look-backs of blocks
  // that advance in lockstep see fewer published prefixes.)
  scan_lookback_kernel<T, kInclusive, TH, CH, sizeof(T) == 4 ? MINB4 : MINB8>
      <<<static_cast<unsigned>(tiles), TH, 0, st>>>(in, out, n, tiles,
                                                     reinterpret_cast<unsigned long long *>(w),
                                                     state, tile_base, tma, vec_out, timeout_ns,
                                                     fault);
  return launch_status();
}

// The chunked reduce-then-scan with slices of kSlice tiles, as one
// cooperative launch; EDPP_ENOMEM (a fallback signal, nothing launched) when
// the kernel cannot be resident on this device or the cooperative launch is
// refused.
template <typename T, bool kInclusive, int kSlice, bool kHint = false>
int launch_rts_chunked(const T *in, T *out, int64_t n, char *w, cudaStream_t st, bool tma,
                       bool vec_out, uint64_t timeout_ns, unsigned *fault) {
  static int cresident[64];
  static std::once_flag conce[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::call_once(conce[dev], [dev] {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, rts_chunked_kernel<T, kInclusive, kSlice, kHint>, kThreads, 0) != cudaSuccess)
      per_sm = 0;
    cresident[dev] = per_sm * device_sm_count();
  });
  if (cresident[dev] <= 0) return EDPP_ENOMEM;
  const int64_t slices = slices_of<T>(n, kSlice);
  const int64_t g = std::min<int64_t>({slices, cresident[dev], kMaxChunkBlocks});
  const int64_t chunks = (slices + g - 1) / g;
  T *sums = reinterpret_cast<T *>(w + kHeader);
  unsigned *cnt = reinterpret_cast<unsigned *>(w + kHeader + chunked_sums_bytes<T>(n));
  if (cudaMemsetAsync(w, 0, kHeader, st) != cudaSuccess ||
      cudaMemsetAsync(cnt, 0, sizeof(unsigned) * static_cast<size_t>(chunks), st) != cudaSuccess)
    return EDPP_ECUDA;
  unsigned *abort_flag = reinterpret_cast<unsigned *>(w + 8);
  int64_t n_arg = n, chunks_arg = chunks;
  bool tma_arg = tma, vec_arg = vec_out;
  uint64_t to_arg = timeout_ns;
  void *args[] = {const_cast<T **>(&in), &out, &n_arg, &chunks_arg, &sums, &cnt, &abort_flag,
                  &tma_arg, &vec_arg, &to_arg, &fault};
  if (cudaLaunchCooperativeKernel(
          reinterpret_cast<const void *>(rts_chunked_kernel<T, kInclusive, kSlice, kHint>),
          dim3(static_cast<unsigned>(g)), dim3(kThreads), args, 0, st) != cudaSuccess) {
    // the grid could not be made co-resident (another context holds SMs):
    // clear the launch error and let the caller take the three-launch form
    cudaGetLastError();
    return EDPP_ENOMEM;
  }
  return launch_status();
}

// variant < 0: the tuning table's choice for this size (else the default).
template <typename T, bool kInclusive>
int scan_impl(const T *in, T *out, int64_t n, int algo, void *ws, size_t ws_bytes, void *stream,
              int64_t tile_base = 0, uint64_t timeout_ns = kDefaultWaitNs, int variant = -1) {
  if (n < 0) return EDPP_EINVAL;
  if (algo != EDPP_SCAN_LOOKBACK && algo != EDPP_SCAN_RTS && algo != EDPP_SCAN_SSA)
    return EDPP_EINVAL;
  if (n == 0) return EDPP_OK;
  if (!in || !out) return EDPP_EINVAL;
  const size_t need = workspace_bytes<T>(n, algo);
  if (!ws || ws_bytes < need) return EDPP_ENOMEM;
  cudaStream_t st = as_stream(stream);
  unsigned *fault = fault_word();
  if (!fault) return EDPP_ECUDA;
  const bool tma = aligned16(in);
  const bool vec_out = aligned16(out);
  char *w = static_cast<char *>(ws);

  if (algo == EDPP_SCAN_LOOKBACK) {
    if (variant < 0) variant = tuned_variant(EDPP_TUNE_SCAN_LOOKBACK, sizeof(T), n, 0);
    switch (variant) {
      case 1:
        return launch_lookback<T, kInclusive, 256, 8, 6, 4>(in, out, n, w, st, tile_base, tma,
                                                            vec_out, timeout_ns, fault);
      case 2:
        return launch_lookback<T, kInclusive, 512, 4, 6, 4>(in, out, n, w, st, tile_base, tma,
                                                            vec_out, timeout_ns, fault);
      case 3:
        return launch_lookback<T, kInclusive, 512, 8, 3, 2>(in, out, n, w, st, tile_base, tma,
                                                            vec_out, timeout_ns, fault);
      default:
        return launch_lookback<T, kInclusive, kLbThreads, kLbChunks, 12, 8>(
            in, out, n, w, st, tile_base, tma, vec_out, timeout_ns, fault);
    }
  }

  int64_t blocks, tpb;
  chunk_grid<T>(n, blocks, tpb);
  T *partials = reinterpret_cast<T *>(w + kHeader);
  const int64_t per = tpb * TS<T>::kTile;
  if (algo == EDPP_SCAN_RTS && variant < 0)
    variant = tuned_variant(EDPP_TUNE_SCAN_RTS, sizeof(T), n, 0);
  if (algo == EDPP_SCAN_RTS && variant != 4 &&
      static_cast<double>(n) * sizeof(T) <= 0.6 * static_cast<double>(device_l2_bytes())) {
    // the input stays in L2 between the reduce and the scan: one launch
    static int resident[64];
    static std::once_flag once[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    std::call_once(once[dev], [dev] {
      int per_sm = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rts_fused_kernel<T, kInclusive>,
                                                        kThreads, 0) != cudaSuccess)
        per_sm = 0;
      resident[dev] = per_sm * device_sm_count();
    });
    if (resident[dev] > 0) {
      const int64_t tiles = tiles_of<T>(n);
      const int64_t g0 = std::min<int64_t>({tiles, resident[dev], kMaxChunkBlocks});
      const int64_t ftpb = (tiles + g0 - 1) / g0;
      const int64_t g = (tiles + ftpb - 1) / ftpb;
      if (cudaMemsetAsync(w, 0, kHeader, st) != cudaSuccess) return EDPP_ECUDA;
      unsigned *ctl = reinterpret_cast<unsigned *>(w);
      int64_t n_arg = n, tpb_arg = ftpb;
      bool tma_arg = tma, vec_arg = vec_out;
      uint64_t to_arg = timeout_ns;
      void *args[] = {const_cast<T **>(&in), &out, &n_arg, &tpb_arg, &partials, &ctl,
                      &tma_arg, &vec_arg, &to_arg, &fault};
      if (cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(rts_fused_kernel<T, kInclusive>),
                                      dim3(static_cast<unsigned>(g)), dim3(kThreads), args, 0,
                                      st) == cudaSuccess)
        return launch_status();
      cudaGetLastError();  // not co-resident: fall through to the other forms
    }
  }
  if (algo == EDPP_SCAN_RTS) {
    // larger than L2: the chunked one-launch form, which reads each element
    // from DRAM once
    int s;
    switch (variant) {
      case 3:
        s = launch_rts_chunked<T, kInclusive, 2, true>(in, out, n, w, st, tma, vec_out, timeout_ns,
                                                       fault);
        break;
      case 1:
        s = launch_rts_chunked<T, kInclusive, 1>(in, out, n, w, st, tma, vec_out, timeout_ns,
                                                 fault);
        break;
      case 2:
        s = launch_rts_chunked<T, kInclusive, 4>(in, out, n, w, st, tma, vec_out, timeout_ns,
                                                 fault);
        break;
      default:
        s = launch_rts_chunked<T, kInclusive, 2>(in, out, n, w, st, tma, vec_out, timeout_ns,
                                                 fault);
    }
    if (s != EDPP_ENOMEM) return s;
    reduce_blocks_kernel<T><<<static_cast<unsigned>(blocks), kThreads, 0, st>>>(in, n, per,
                                                                                partials, tma);
    scan_partials_kernel<T><<<1, 1024, 0, st>>>(partials, static_cast<int>(blocks));
    scan_blocks_kernel<T, kInclusive, true><<<static_cast<unsigned>(blocks), kThreads, 0, st>>>(
        in, out, n, tpb, partials, nullptr, tma, vec_out, timeout_ns, fault);
  } else {  // SSA
    scan_blocks_kernel<T, kInclusive, false><<<static_cast<unsigned>(blocks), kThreads, 0, st>>>(
        in, out, n, tpb, nullptr, partials, tma, vec_out, timeout_ns, fault);
    scan_partials_kernel<T><<<1, 1024, 0, st>>>(partials, static_cast<int>(blocks));
    add_offsets_kernel<T><<<static_cast<unsigned>(blocks), kThreads, 0, st>>>(out, n, per,
                                                                             partials, vec_out);
  }
  return launch_status();
}

}  // namespace

int scan_with_variant(const void *in, void *out, int64_t length, int elem_bytes, int algo,
                      int variant, void *ws, size_t ws_bytes, void *stream) {
  if (variant < 0 || variant >= scan_variants(algo)) return EDPP_EINVAL;
  if (elem_bytes == 4)
    return scan_impl<int32_t, false>(static_cast<const int32_t *>(in), static_cast<int32_t *>(out),
                                     length, algo, ws, ws_bytes, stream, 0, kDefaultWaitNs,
                                     variant);
  if (elem_bytes == 8)
    return scan_impl<int64_t, false>(static_cast<const int64_t *>(in), static_cast<int64_t *>(out),
                                     length, algo, ws, ws_bytes, stream, 0, kDefaultWaitNs,
                                     variant);
  return EDPP_EINVAL;
}

int scan_variants(int algo) {
  return algo == EDPP_SCAN_LOOKBACK ? kLbVariants : algo == EDPP_SCAN_RTS ? kRtsVariants : 0;
}

}  // namespace edpp

extern "C" {

size_t edpp_scan_workspace_size(int64_t length, int dtype, int algo) {
  switch (dtype) {
    case EDPP_I32: return edpp::workspace_bytes<int32_t>(length, algo);
    case EDPP_I64: return edpp::workspace_bytes<int64_t>(length, algo);
    case EDPP_F32: return edpp::workspace_bytes<float>(length, algo);
    default: return 0;
  }
}

int edpp_scan_exclusive_i32(const int32_t *in, int32_t *out, int64_t length, int algo, void *ws,
                            size_t ws_bytes, void *stream) {
  return edpp::scan_impl<int32_t, false>(in, out, length, algo, ws, ws_bytes, stream);
}
int edpp_scan_inclusive_i32(const int32_t *in, int32_t *out, int64_t length, int algo, void *ws,
                            size_t ws_bytes, void *stream) {
  return edpp::scan_impl<int32_t, true>(in, out, length, algo, ws, ws_bytes, stream);
}
int edpp_scan_exclusive_i64(const int64_t *in, int64_t *out, int64_t length, int algo, void *ws,
                            size_t ws_bytes, void *stream) {
  return edpp::scan_impl<int64_t, false>(in, out, length, algo, ws, ws_bytes, stream);
}
int edpp_scan_inclusive_i64(const int64_t *in, int64_t *out, int64_t length, int algo, void *ws,
                            size_t ws_bytes, void *stream) {
  return edpp::scan_impl<int64_t, true>(in, out, length, algo, ws, ws_bytes, stream);
}
int edpp_scan_exclusive_f32(const float *in, float *out, int64_t length, int algo, void *ws,
                            size_t ws_bytes, void *stream) {
  return edpp::scan_impl<float, false>(in, out, length, algo, ws, ws_bytes, stream);
}
int edpp_scan_inclusive_f32(const float *in, float *out, int64_t length, int algo, void *ws,
                            size_t ws_bytes, void *stream) {
  return edpp::scan_impl<float, true>(in, out, length, algo, ws, ws_bytes, stream);
}

int edpp_selftest_lookback_timeout(const int32_t *in, int32_t *out, int64_t length,
                                   uint64_t timeout_ns, void *ws, size_t ws_bytes, void *stream) {
  if (length <= 0 || timeout_ns == 0) return EDPP_EINVAL;
  // Tickets start at tile 1: tile 0 is never scanned, so tile 1 (and every
  // later tile) waits for a prefix nobody publishes until the limit runs out.
  return edpp::scan_impl<int32_t, false>(in, out, length, EDPP_SCAN_LOOKBACK, ws, ws_bytes, stream,
                                         /*tile_base=*/1, timeout_ns, /*variant=*/0);
}

}  // extern "C"

// ---- allocation-free exclusive scan -------------------------------------------
// For callers that cannot allocate device memory: a host thread that must
// not enter the device allocator (a real-time loop that cannot afford its
// latency or its implicit synchronisation), or a plugin whose host
// application owns every device allocation and hands it only the arrays it
// works on.  The look-back state lives in this file-scope
// device array instead of a caller workspace.  Each GPU that loads the library
// holds the array until the process exits.
namespace edpp {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(1) << 20;  // 1 MiB per device
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Largest length the scratch array can serve: the header plus 8 bytes of
// look-back state per tile of TS<int32_t>::kTile elements.
constexpr int64_t kNoAllocMaxLength =
    static_cast<int64_t>((kNoAllocScratchBytes - kHeader) / 8) * TS<int32_t>::kTile;

constexpr int kMaxDev = 64;
std::once_flag g_noalloc_once[kMaxDev];
void *g_noalloc_ptr[kMaxDev];
cudaError_t g_noalloc_err[kMaxDev];

// Device address of the scratch array on the current device.  In host code
// the symbol is only a stand-in, never a usable device address, so it is
// resolved with cudaGetSymbolAddress once per device, with that device
// current.
void *noalloc_scratch(cudaError_t &err) {
  int dev = 0;
  err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return nullptr;
  if (dev < 0 || dev >= kMaxDev) {
    err = cudaErrorInvalidDevice;
    return nullptr;
  }
  std::call_once(g_noalloc_once[dev], [dev] {
    void *p = nullptr;
    g_noalloc_err[dev] = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    g_noalloc_ptr[dev] = g_noalloc_err[dev] == cudaSuccess ? p : nullptr;
  });
  err = g_noalloc_err[dev];
  return g_noalloc_ptr[dev];
}

}  // namespace
}  // namespace edpp

extern "C" {

int64_t edpp_scan_exclusive_i32_noalloc_max_length(void) { return edpp::kNoAllocMaxLength; }

int edpp_scan_exclusive_i32_noalloc(const int32_t *in, int32_t *out, int64_t length,
                                    void *stream) {
  using namespace edpp;
  if (length < 0) return EDPP_EINVAL;
  if (length > kNoAllocMaxLength) return EDPP_EINVAL;  // beyond the static scratch
  if (length == 0) return EDPP_OK;
  if (!in || !out) return EDPP_EINVAL;
  cudaError_t err;
  char *w = static_cast<char *>(noalloc_scratch(err));
  if (!w) return EDPP_ECUDA;
  unsigned *fault = fault_word();
  if (!fault) return EDPP_ECUDA;
  cudaStream_t st = as_stream(stream);
  const int64_t tiles = tiles_of<int32_t>(length);
  // The array keeps the previous call's contents: clear the ticket, the
  // abort flag and this call's look-back state before the launch.
  const size_t used = kHeader + LookbackState<int32_t>::bytes(tiles);
  if (cudaMemsetAsync(w, 0, used, st) != cudaSuccess) return EDPP_ECUDA;
  LookbackState<int32_t> state;
  state.bind(w + kHeader, tiles);
  scan_lookback_kernel<int32_t, false><<<static_cast<unsigned>(tiles), kLbThreads, 0, st>>>(
      in, out, length, tiles, reinterpret_cast<unsigned long long *>(w), state, 0,
      aligned16(in), aligned16(out), kDefaultWaitNs, fault);
  return launch_status();
}

}  // extern "C"
