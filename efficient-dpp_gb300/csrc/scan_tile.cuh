// scan_tile.cuh — block-level tile scan and the decoupled look-back state
// shared by the global scans (scan.cu) and the batched kernel (batch.cu).
//
// Tile layout ("row-striped 16-byte chunks"): a tile of kTile elements is cut
// into 16-byte chunks of E = 16/sizeof(T) elements; thread t of a block of
// THREADS owns chunks t, t+THREADS, ..., t+(CHUNKS-1)*THREADS.  Every chunk
// access of a warp is then one contiguous 512-byte segment, so global loads
// and stores are fully coalesced 128-bit accesses and shared-memory accesses
// are free of bank conflicts, with no transpose.  The prefix order is
// (row k, thread t, element e); a warp scans its CHUNKS chunk sums at once
// and one warp scans the WARPS*CHUNKS = 32 warp totals.
#pragma once

#include "common.cuh"

namespace edpp {

// ---- wrapping arithmetic ----------------------------------------------------
// Integer prefix sums wrap in two's complement, bit-identical to the
// reference's int scans compiled with wrapping semantics.
__device__ __forceinline__ int32_t op_add(int32_t a, int32_t b) {
  return static_cast<int32_t>(static_cast<uint32_t>(a) + static_cast<uint32_t>(b));
}
__device__ __forceinline__ int64_t op_add(int64_t a, int64_t b) {
  return static_cast<int64_t>(static_cast<uint64_t>(a) + static_cast<uint64_t>(b));
}
__device__ __forceinline__ float op_add(float a, float b) { return a + b; }

template <typename T> __device__ __forceinline__ T zero_of() { return T(0); }

template <typename T> __device__ __forceinline__ T shfl_up(T v, int d) {
  return __shfl_up_sync(0xffffffffu, v, d);
}
template <typename T> __device__ __forceinline__ T shfl_idx(T v, int l) {
  return __shfl_sync(0xffffffffu, v, l);
}
template <typename T> __device__ __forceinline__ T shfl_xor(T v, int m) {
  return __shfl_xor_sync(0xffffffffu, v, m);
}

// Inclusive warp scan.
template <typename T> __device__ __forceinline__ T warp_incl_scan(T x, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T y = shfl_up(x, d);
    if (lane >= d) x = op_add(x, y);
  }
  return x;
}

// Warp sum (every lane gets the total).
template <typename T> __device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) x = op_add(x, shfl_xor(x, m));
  return x;
}

// 16 bytes of T.
template <typename T> union Chunk {
  static constexpr int E = 16 / static_cast<int>(sizeof(T));
  uint4 raw;
  T e[16 / sizeof(T)];
};

// ---- decoupled look-back tile state ---------------------------------------
// Flags: 0 = not yet published (the workspace is zeroed before each call),
// 1 = aggregate of the tile alone, 2 = inclusive prefix through the tile.
constexpr uint32_t kFlagNone = 0, kFlagAgg = 1, kFlagIncl = 2;

template <typename T, bool kPacked = (sizeof(T) == 4)> struct LookbackState;

// 32-bit values: flag and value share one 64-bit word, written and read with
// single-copy-atomic 64-bit accesses.
template <typename T> struct LookbackState<T, true> {
  uint64_t *words;
  static size_t bytes(int64_t tiles) { return round_up(static_cast<size_t>(tiles) * 8, 256); }
  __host__ __device__ void bind(void *p, int64_t /*tiles*/) { words = static_cast<uint64_t *>(p); }
  __device__ __forceinline__ void publish(int64_t tile, uint32_t flag, T v) const {
    uint32_t bits;
    memcpy(&bits, &v, 4);
    st_relaxed_u64(words + tile, (static_cast<uint64_t>(flag) << 32) | bits);
  }
  __device__ __forceinline__ void read(int64_t tile, uint32_t &flag, T &v) const {
    const uint64_t w = ld_relaxed_u64(words + tile);
    flag = static_cast<uint32_t>(w >> 32);
    const uint32_t bits = static_cast<uint32_t>(w);
    memcpy(&v, &bits, 4);
  }
};

// 64-bit values: two 64-bit words per tile, {flag, low half} and {flag, high
// half}, each written and read single-copy atomically (one round trip for a
// read, like the 32-bit form).  A reader that sees different flags in the
// two words caught a tile between its aggregate and its inclusive prefix and
// reports "not yet published", so it reads again.
template <typename T> struct LookbackState<T, false> {
  uint64_t *words;
  static size_t bytes(int64_t tiles) { return round_up(static_cast<size_t>(tiles) * 16, 256); }
  __host__ __device__ void bind(void *p, int64_t /*tiles*/) { words = static_cast<uint64_t *>(p); }
  __device__ __forceinline__ void publish(int64_t tile, uint32_t flag, T v) const {
    uint64_t bits;
    memcpy(&bits, &v, 8);
    const uint64_t f = static_cast<uint64_t>(flag) << 32;
    st_relaxed_u64(words + 2 * tile, f | (bits & 0xffffffffull));
    st_relaxed_u64(words + 2 * tile + 1, f | (bits >> 32));
  }
  __device__ __forceinline__ void read(int64_t tile, uint32_t &flag, T &v) const {
    const uint64_t lo = ld_relaxed_u64(words + 2 * tile);
    const uint64_t hi = ld_relaxed_u64(words + 2 * tile + 1);
    const uint32_t f0 = static_cast<uint32_t>(lo >> 32), f1 = static_cast<uint32_t>(hi >> 32);
    flag = f0 == f1 ? f0 : kFlagNone;
    const uint64_t bits = (hi << 32) | (lo & 0xffffffffull);
    memcpy(&v, &bits, 8);
  }
};

// Look-back by one full warp for tile `tile` (> 0) whose aggregate is `agg`.
// Returns the exclusive prefix of the tile (every lane).  Publishes the
// aggregate first and the inclusive prefix last.  Every wait is bounded by
// timeout_ns; on timeout it raises EDPP_FAULT_TIMEOUT in the device fault
// word, sets the call's `abort_flag` (so the other waiting blocks of the same
// call give up at once), sets `ok` false and returns without publishing the
// inclusive prefix.  `abort_flag` lives in the call's zeroed workspace, so a
// fault of an earlier call never affects this one.
template <typename T, typename State>
__device__ __forceinline__ T lookback_warp(const State &st, int64_t tile, T agg, int lane,
                                           uint64_t timeout_ns, unsigned *fault,
                                           unsigned *abort_flag, bool &ok) {
  if (lane == 0) st.publish(tile, kFlagAgg, agg);
  T excl = zero_of<T>();
  int64_t hi = tile - 1;  // nearest predecessor of the current window
  uint64_t t0 = 0;
  ok = true;
  while (true) {
    const int64_t idx = hi - lane;
    uint32_t f = kFlagIncl;
    T v = zero_of<T>();
    if (idx >= 0) st.read(idx, f, v);
    // Wait until every lane up to the nearest inclusive prefix is published.
    while (true) {
      const unsigned pmask = __ballot_sync(0xffffffffu, f == kFlagIncl);
      const unsigned xmask = __ballot_sync(0xffffffffu, f == kFlagNone);
      const int low = pmask ? (__ffs(pmask) - 1) : 31;
      const unsigned need = (low >= 31) ? 0xffffffffu : ((2u << low) - 1u);
      if ((xmask & need) == 0u) break;
      if (t0 == 0) t0 = globaltimer_ns();
      const bool expired = (globaltimer_ns() - t0 > timeout_ns) || fault_raised(abort_flag);
      if (__any_sync(0xffffffffu, expired)) {  // warp-uniform exit
        if (lane == 0) {
          raise_fault(fault, EDPP_FAULT_TIMEOUT);
          atomicOr(abort_flag, 1u);
        }
        ok = false;
        return excl;
      }
      __nanosleep(64);
      if (f == kFlagNone && idx >= 0) st.read(idx, f, v);
    }
    const unsigned pmask = __ballot_sync(0xffffffffu, f == kFlagIncl);
    if (pmask) {
      const int low = __ffs(pmask) - 1;
      excl = op_add(excl, warp_sum(lane <= low ? v : zero_of<T>()));
      break;
    }
    excl = op_add(excl, warp_sum(v));
    hi -= 32;
  }
  if (lane == 0) st.publish(tile, kFlagIncl, op_add(excl, agg));
  return excl;
}

// ---- block tile scan --------------------------------------------------------
template <typename T, int THREADS, int CHUNKS> struct TileScan {
  static constexpr int E = Chunk<T>::E;
  static constexpr int WARPS = THREADS / 32;
  static constexpr int kTile = THREADS * CHUNKS * E;
  static constexpr int NT = WARPS * CHUNKS;  // warp totals of a tile
  static constexpr int PER = NT / 32;        // warp totals per lane of warp 0
  static_assert(NT == 32 || NT == 64 || NT == 128, "one warp scans the warp totals");

  struct Shared {
    T warp_tot[NT];  // [k*WARPS + w] inclusive total of warp w in row k
    T warp_pre[NT];  // exclusive tile prefix of (row k, warp w)
    T prefix;        // exclusive prefix of the whole tile
    T total;         // tile aggregate
  };

  // Phase 1: load this thread's chunks from shared memory, scan them in
  // place (inclusive within chunk), compute the warp-exclusive chunk offsets
  // and publish warp totals.  Caller then __syncthreads().
  __device__ __forceinline__ static void phase1(const T *tile_smem, Chunk<T> (&c)[CHUNKS],
                                                T (&warp_excl)[CHUNKS], Shared &sh) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    T incl[CHUNKS];
#pragma unroll
    for (int k = 0; k < CHUNKS; ++k) {
      c[k].raw = reinterpret_cast<const uint4 *>(tile_smem)[k * THREADS + t];
#pragma unroll
      for (int e = 1; e < E; ++e) c[k].e[e] = op_add(c[k].e[e - 1], c[k].e[e]);
      incl[k] = c[k].e[E - 1];
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
      for (int k = 0; k < CHUNKS; ++k) {
        const T y = shfl_up(incl[k], d);
        if (lane >= d) incl[k] = op_add(incl[k], y);
      }
    }
#pragma unroll
    for (int k = 0; k < CHUNKS; ++k) {
      const T ex = shfl_up(incl[k], 1);
      warp_excl[k] = lane == 0 ? zero_of<T>() : ex;
      if (lane == 31) sh.warp_tot[k * WARPS + w] = incl[k];
    }
  }

  // Phase 2 (warp 0 only, after the barrier): scan the NT warp totals, PER
  // consecutive ones per lane.  Returns the tile aggregate in every lane.
  __device__ __forceinline__ static T phase2_warp0(Shared &sh, int lane) {
    T x[PER];
    T s = zero_of<T>();
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      x[i] = sh.warp_tot[lane * PER + i];
      s = op_add(s, x[i]);
    }
    const T xi = warp_incl_scan(s, lane);
    const T ex = shfl_up(xi, 1);
    T run = lane == 0 ? zero_of<T>() : ex;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      sh.warp_pre[lane * PER + i] = run;
      run = op_add(run, x[i]);
    }
    return shfl_idx(xi, 31);
  }

  // Phase 3: final values.  `prefix` = exclusive prefix of the tile.
  // Inclusive: element value = prefix + chunk offset + inclusive-in-chunk.
  // Exclusive: shifts the in-chunk scan by one.
  template <bool kInclusive>
  __device__ __forceinline__ static void phase3(Chunk<T> (&c)[CHUNKS],
                                                const T (&warp_excl)[CHUNKS], const Shared &sh,
                                                T prefix) {
    const int w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < CHUNKS; ++k) {
      const T base = op_add(prefix, op_add(sh.warp_pre[k * WARPS + w], warp_excl[k]));
      if (kInclusive) {
#pragma unroll
        for (int e = 0; e < E; ++e) c[k].e[e] = op_add(base, c[k].e[e]);
      } else {
#pragma unroll
        for (int e = E - 1; e >= 1; --e) c[k].e[e] = op_add(base, c[k].e[e - 1]);
        c[k].e[0] = base;
      }
    }
  }

  // Store this thread's chunks to out[tile_base ...], `count` valid elements
  // in the tile.  vec: out is 16-byte aligned.  kStream: evict-first stores.
  template <bool kStream = false>
  __device__ __forceinline__ static void store(T *out, int64_t tile_base, int count,
                                               const Chunk<T> (&c)[CHUNKS], bool vec) {
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < CHUNKS; ++k) {
      const int off = (k * THREADS + t) * E;
      if (vec && off + E <= count) {
        uint4 *dst = reinterpret_cast<uint4 *>(out + tile_base) + k * THREADS + t;
        if (kStream) __stcs(dst, c[k].raw);
        else *dst = c[k].raw;
      } else {
#pragma unroll
        for (int e = 0; e < E; ++e)
          if (off + e < count) out[tile_base + off + e] = c[k].e[e];
      }
    }
  }
};

// Stage tile elements [0,count) of `src` (global) into `dst` (shared),
// zero-filling [count, kTile).  When `tma` (src 16-byte aligned), the
// 16-byte-multiple prefix goes by one bulk copy signalled on `bar`
// (issued by thread 0) and the rest by plain loads.  Returns the number of
// bytes in flight on `bar` (0 if none); the caller waits on `bar` and then
// __syncthreads() before reading.
// kLastUse: the tile's bytes are read for the last time, so the bulk copy
// carries an evict-first L2 hint (`policy` from l2_policy_evict_first).
template <typename T, int kTile, int THREADS, bool kLastUse = false>
__device__ __forceinline__ uint32_t stage_tile(T *dst, const T *src, int count, bool tma,
                                               uint64_t *bar, uint64_t policy = 0) {
  uint32_t bulk = 0;
  if (tma) bulk = (static_cast<uint32_t>(count) * sizeof(T)) & ~15u;
  if (threadIdx.x == 0 && bulk) {
    mbar_arrive_expect_tx(bar, bulk);
    if (kLastUse) tma_load_1d_evict_first(dst, src, bulk, bar, policy);
    else tma_load_1d(dst, src, bulk, bar);
  }
  const int first = static_cast<int>(bulk / sizeof(T));
  if (first < kTile) {
    for (int i = first + threadIdx.x; i < kTile; i += THREADS) dst[i] = i < count ? src[i] : zero_of<T>();
  }
  return bulk;
}

}  // namespace edpp
