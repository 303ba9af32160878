// split.cu — stable multi-split of int32 keys (KO), key/value arrays
// (KVS_SOA) or {key,value} pairs (KVS_AOS) by bucket = key & (B-1).
//
// Same three stages as the reference's split (histogram -> scan of the
// bucket-major histogram -> shuffle; opencl/primitives/splitImpl.cpp:66-140,
// cuda/test_split.cu:149-186), re-planned for GB300:
//
//  1. hist:    one block per tile of kTile elements counts its buckets with
//              shared-memory atomics (one per element) and
//              writes column t of the bucket-major matrix his[b*T + t], the
//              layout of WI/WG_histogram (split_kernel.cl:370,451) and of
//              warp_histogram (cuda/test_split.cu:48).
//  2. scan:    exclusive look-back scan of his[] in place (scan.cu), as the
//              reference runs scan_chained(d_his, d_his, ...) in place
//              (splitImpl.cpp:97).  his[b*T + t] is then the first output
//              index of bucket b's elements from tile t.
//  3. scatter: one block per tile stages the tile in shared memory by TMA
//              bulk copy; every warp ranks its contiguous 1/WARPS of the tile
//              in input order (rank = popc of the lower lanes in the
//              element's peer group + the warp's running count of the
//              bucket; the peer group from votes on the bucket bits up to 4
//              buckets, from a per-warp lane mask per bucket up to 256, from
//              a leader table plus votes above); ranks of all warps are
//              combined per bucket, the tile is re-laid out in shared memory
//              in bucket order, and written out as one contiguous run per
//              bucket (coalesced), at his[b*T + t] + rank.
//
// Ranks follow input order inside a warp segment, warp segments follow
// input order inside a tile, tiles follow input order in the scan: the split
// is stable, bit-identical to single_split (split_kernel.cl:676-736),
// WG_split with FIXED_REORDER and the CUDA pre_scan/post_scan split.  There
// are no inter-block waits.
#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace edpp {
namespace {

constexpr int kTile = 8192;
constexpr int kMaxBuckets = 8192;     // public limit; from 2048 on, two passes
constexpr int kOnePassMax = 1024;     // largest bucket count one pass takes
constexpr int kHistThreads = 512;
constexpr int kDirectBuckets = 2;  // up to this many buckets the scatter writes from registers
// Up to this many bucket bits, each lane keeps one bucket's warp count in a
// register; above, counts live in shared memory behind a peer table.
// Measured at 2^28 pairs (same process, both builds), against the lane-mask
// table: 2 against 3 bits, 8 buckets 1.27 -> 1.12 ms, the others even; 1
// bit made 4 buckets 5% slower.
constexpr int kRegBits = 2;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Key of element i.
template <int LAYOUT> __device__ __forceinline__ int32_t key_at(const int32_t *k, int64_t i) {
  return LAYOUT == EDPP_KVS_AOS ? k[2 * i] : k[i];
}

// ---- stage 1: per-tile bucket counts ----------------------------------------
template <int LAYOUT>
__global__ void __launch_bounds__(kHistThreads)
    split_hist_kernel(const int32_t *__restrict__ keys, int64_t n, int buckets, int shift,
                      int64_t tiles, int32_t *__restrict__ his, bool vec) {
  __shared__ uint32_t cnt[kOnePassMax];
  const unsigned mask = static_cast<unsigned>(buckets - 1);
  for (int b = threadIdx.x; b < buckets; b += kHistThreads) cnt[b] = 0;
  __syncthreads();
  const int64_t t = blockIdx.x;
  const int64_t base = t * kTile;
  const int count = static_cast<int>(min64(kTile, n - base));

  auto add = [&](bool valid, int32_t key) {
    if (valid) atomicAdd(&cnt[(static_cast<unsigned>(key) >> shift) & mask], 1u);
  };

  if (LAYOUT != EDPP_KVS_AOS && vec && count == kTile) {
    // 16-byte vectors, warp-contiguous: 4 keys per thread per step.
    const int4 *k4 = reinterpret_cast<const int4 *>(keys + base);
#pragma unroll 2
    for (int v = threadIdx.x; v < kTile / 4; v += kHistThreads) {
      const int4 q = __ldcs(k4 + v);
      add(true, q.x);
      add(true, q.y);
      add(true, q.z);
      add(true, q.w);
    }
  } else if (LAYOUT == EDPP_KVS_AOS && vec && count == kTile) {
    // 16-byte vectors of two pairs.
    const int4 *p4 = reinterpret_cast<const int4 *>(keys + 2 * base);
#pragma unroll 2
    for (int v = threadIdx.x; v < kTile / 2; v += kHistThreads) {
      const int4 q = __ldcs(p4 + v);
      add(true, q.x);
      add(true, q.z);
    }
  } else {
    for (int i0 = 0; i0 < count; i0 += kHistThreads) {
      const int i = i0 + threadIdx.x;
      const bool valid = i < count;
      add(valid, valid ? key_at<LAYOUT>(keys, base + i) : 0);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < buckets; b += kHistThreads)
    his[static_cast<int64_t>(b) * tiles + t] = static_cast<int32_t>(cnt[b]);
}

// ---- stage 3: stable scatter --------------------------------------------------
template <int THREADS> struct ScatterCfg {
  static constexpr int kWarps = THREADS / 32;
  static constexpr int kSeg = kTile / kWarps;  // elements per warp
  static constexpr int kIters = kSeg / 32;     // per lane
};

// Bucket runs written by bulk copies (KO and KVS_SOA, 3 to kBulkBuckets
// buckets, 16-byte-aligned outputs): each staging array then holds
// stage_len(buckets) elements, the tile plus up to 3 spare slots per bucket
// so that a run's staging start can share its output start's residue mod 4.
// Measured at 2^28 pairs against the per-element write-out (same process,
// both builds): 4 / 8 / 16 buckets 9 / 7 / 4% faster; from 32 buckets on,
// with runs of 256 elements or fewer, 3-14% slower.
constexpr int kBulkBuckets = 16;
__host__ __device__ constexpr int stage_len(int buckets, bool bulk) {
  return kTile + (bulk ? (3 * buckets + 3) / 4 * 4 : 0);
}

// Peer table of the ranking, per warp: from kRegBits + 1 to 8 bucket bits one
// 32-bit lane mask per bucket (lanes OR themselves in); above 8 bits one
// leader byte per value of the low 8 bucket bits.
__host__ __device__ constexpr int peer_table_bytes(int buckets) {
  return buckets <= 256 ? 4 * buckets : 256;
}

// Dynamic shared memory of the scatter kernel.
template <int THREADS, int LAYOUT> size_t scatter_smem_bytes(int buckets, bool bulk = false) {
  const size_t stage = (LAYOUT == EDPP_KO) ? 4 * static_cast<size_t>(stage_len(buckets, bulk))
                       : (LAYOUT == EDPP_KVS_SOA) ? 8 * static_cast<size_t>(stage_len(buckets, bulk))
                                                  : kTile * 8;
  return stage + round_up(static_cast<size_t>(ScatterCfg<THREADS>::kWarps) * buckets * 2, 16) +
         2 * static_cast<size_t>(buckets) * 4 +
         static_cast<size_t>(ScatterCfg<THREADS>::kWarps) * peer_table_bytes(buckets);
}

// Two blocks per SM (their staging fills shared memory): at most 64 registers.
// kWide: more than 256 buckets, ranked through the leader table; up to 256
// buckets the register counts and lane masks.  Two kernels rather than one
// carrying every form: 16 / 32 / 64 / 256 buckets 19 / 14 / 12 / 7% faster
// at 2^28 pairs, 512 and 1024 even (one process, both builds).  A third
// kernel for the register counts alone spilled and made 2 buckets 4% slower.
template <int THREADS, int LAYOUT, bool kWide>
__global__ void __launch_bounds__(THREADS, 2)
    split_scatter_kernel(const int32_t *__restrict__ keys_in, int32_t *__restrict__ keys_out,
                         const int32_t *__restrict__ vals_in, int32_t *__restrict__ vals_out,
                         int64_t n, int buckets, int shift, int64_t tiles,
                         const int32_t *__restrict__ his, bool tma, bool bulk,
                         uint64_t timeout_ns, unsigned *fault) {
  using C = ScatterCfg<THREADS>;
  extern __shared__ __align__(128) unsigned char smem[];
  // Layout: stage (keys[L] + vals[L] with L = stage_len, or pairs[kTile]) |
  // cnt16 | toff | gofs | peer tables.  `bulk` (KO / SOA only): runs go out by
  // bulk copies.
  const int slen = stage_len(buckets, bulk);
  int32_t *s_keys = reinterpret_cast<int32_t *>(smem);
  int32_t *s_vals = s_keys + slen;  // SOA only
  int2 *s_pairs = reinterpret_cast<int2 *>(smem);  // AOS only
  const size_t stage = LAYOUT == EDPP_KO ? 4 * static_cast<size_t>(slen)
                       : LAYOUT == EDPP_KVS_SOA ? 8 * static_cast<size_t>(slen) : kTile * 8;
  uint16_t *cnt16 = reinterpret_cast<uint16_t *>(smem + stage);
  int32_t *toff = reinterpret_cast<int32_t *>(
      smem + stage + round_up(static_cast<size_t>(C::kWarps) * buckets * 2, 16));
  int32_t *gofs = toff + buckets;
  unsigned char *s_peer = reinterpret_cast<unsigned char *>(gofs + buckets);  // [kWarps][table]
  __shared__ alignas(8) uint64_t bar;

  const int64_t t = blockIdx.x;
  const int64_t base = t * kTile;
  const int count = static_cast<int>(min64(kTile, n - base));
  const unsigned mask = static_cast<unsigned>(buckets - 1);
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;

  // -- load the tile (bulk copies for the 16-byte-aligned prefix) --
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t bulk_elems = 0;
  if (tma) bulk_elems = (LAYOUT == EDPP_KVS_AOS) ? (count & ~1) : (count & ~3);
  if (tid == 0 && bulk_elems) {
    if (LAYOUT == EDPP_KVS_AOS) {
      mbar_arrive_expect_tx(&bar, bulk_elems * 8);
      tma_load_1d(s_pairs, keys_in + 2 * base, bulk_elems * 8, &bar);
    } else if (LAYOUT == EDPP_KVS_SOA) {
      mbar_arrive_expect_tx(&bar, bulk_elems * 8);
      tma_load_1d(s_keys, keys_in + base, bulk_elems * 4, &bar);
      tma_load_1d(s_vals, vals_in + base, bulk_elems * 4, &bar);
    } else {
      mbar_arrive_expect_tx(&bar, bulk_elems * 4);
      tma_load_1d(s_keys, keys_in + base, bulk_elems * 4, &bar);
    }
  }
  for (int i = static_cast<int>(bulk_elems) + tid; i < count; i += THREADS) {
    if (LAYOUT == EDPP_KVS_AOS) {
      s_pairs[i] = make_int2(keys_in[2 * (base + i)], keys_in[2 * (base + i) + 1]);
    } else {
      s_keys[i] = keys_in[base + i];
      if (LAYOUT == EDPP_KVS_SOA) s_vals[i] = vals_in[base + i];
    }
  }
  for (int i = tid; i < C::kWarps * buckets; i += THREADS) cnt16[i] = 0;
  if (!kWide && buckets > (1 << kRegBits))  // the lane masks start empty
    for (int i = tid; i < C::kWarps * buckets; i += THREADS)
      reinterpret_cast<uint32_t *>(s_peer)[i] = 0u;
  // This thread's buckets for the per-bucket combine below; the first
  // kHisPre of their global run starts (his[b*T + t], one 32-byte sector
  // each) are loaded now, so the round trip overlaps the tile's ranking.
  const int per = (buckets + THREADS - 1) / THREADS;
  const int b_lo = min(buckets, tid * per), b_hi = min(buckets, b_lo + per);
  constexpr int kHisPre = THREADS >= 512 ? 2 : 4;  // 512 threads serve up to 1024 buckets
  int32_t his_pre[kHisPre];
#pragma unroll
  for (int k = 0; k < kHisPre; ++k)
    his_pre[k] = b_lo + k < b_hi ? __ldg(his + static_cast<int64_t>(b_lo + k) * tiles + t) : 0;
  if (bulk_elems) {
    if (!mbar_wait_bounded(&bar, 0, timeout_ns, fault)) return;
  }
  __syncthreads();

  // -- rank: warp w owns tile positions [w*kSeg, (w+1)*kSeg), in order --
  const unsigned lt = lanemask_lt();
  const int kbits = 31 - __clz(buckets);
  uint16_t *my_cnt = cnt16 + w * buckets;
  uint32_t *my_or = reinterpret_cast<uint32_t *>(s_peer) + w * buckets;  // up to 8 bits
  uint8_t *my_last = s_peer + w * 256;                                  // above 8 bits
  int32_t kk[C::kIters];
  int32_t vv[C::kIters];
  uint32_t rk[(C::kIters + 1) / 2];  // two 16-bit ranks per register
  // Up to 2^kRegBits buckets: lane L keeps the warp's running count of bucket
  // L in a register; the per-bit votes give both this lane's group and bucket
  // L's group, so the loop needs no shared memory and no warp barriers.
  uint32_t lane_cnt = 0;
#pragma unroll
  for (int it = 0; it < C::kIters; ++it) {
    const int pos = w * C::kSeg + it * 32 + lane;
    const bool valid = pos < count;
    int32_t key = 0, val = 0;
    if (valid) {
      if (LAYOUT == EDPP_KVS_AOS) {
        const int2 p = s_pairs[pos];
        key = p.x;
        val = p.y;
      } else {
        key = s_keys[pos];
        if (LAYOUT == EDPP_KVS_SOA) val = s_vals[pos];
      }
    }
    const int b = valid ? static_cast<int>((static_cast<unsigned>(key) >> shift) & mask) : -1;
    const unsigned vmask = __ballot_sync(0xffffffffu, valid);
    if (!kWide && kbits <= kRegBits) {
      unsigned peers = vmask, mine = vmask;
      for (int i = 0; i < kbits; ++i) {
        const unsigned bb = __ballot_sync(0xffffffffu, (b >> i) & 1);
        peers &= ((b >> i) & 1) ? bb : ~bb;
        mine &= ((lane >> i) & 1) ? bb : ~bb;  // the lanes holding bucket `lane`
      }
      const uint32_t before = __shfl_sync(0xffffffffu, lane_cnt, b & 31);
      if (lane < buckets) lane_cnt += __popc(mine);
      kk[it] = key;
      vv[it] = val;
      const uint32_t r = valid ? before + __popc(peers & lt) : 0u;
      if (it & 1) rk[it >> 1] |= r << 16;
      else rk[it >> 1] = r;
      continue;
    }
    unsigned peers;
    if (!kWide) {
      // every lane ORs its bit into its bucket's mask: the mask read back is
      // the lane's peer group (2^28 pairs against the leader table below,
      // in one kernel with it: 32 / 64 / 256 buckets 6 / 5 / 2% faster)
      if (valid) atomicOr(&my_or[b], 1u << lane);
      __syncwarp();
      peers = valid ? my_or[b] : 0u;
    } else {
      // the lanes sharing the low 8 bucket bits agree on one leader lane
      // (whichever write lands), 5 votes on the leader's lane number find
      // that group, and one vote per bucket bit above the 8th splits it
      // (a lane-mask table of all buckets would halve the blocks per SM)
      if (valid) my_last[b & 255] = static_cast<uint8_t>(lane);
      __syncwarp();
      peers = match_low_bits(valid ? my_last[b & 255] : 0u, 5, vmask);
      peers &= match_low_bits(static_cast<unsigned>(b) >> 8, kbits - 8, vmask);
    }
    const unsigned lower = peers & lt;
    const uint16_t before = valid ? my_cnt[b] : 0;
    __syncwarp();
    if (valid && lower == 0u) {
      my_cnt[b] = static_cast<uint16_t>(before + __popc(peers));
      if (!kWide) my_or[b] = 0u;  // the group's lowest lane empties the mask
    }
    __syncwarp();
    kk[it] = key;
    vv[it] = val;
    const uint32_t r = static_cast<uint32_t>(before + __popc(lower));
    if (it & 1) rk[it >> 1] |= r << 16;
    else rk[it >> 1] = r;
  }
  if (!kWide && kbits <= kRegBits && lane < buckets) my_cnt[lane] = static_cast<uint16_t>(lane_cnt);
  __syncthreads();

  // -- per bucket: tile count, tile offset, then each warp's first slot --
  // Thread-consecutive buckets so the block-wide scan over buckets is a
  // per-thread serial scan plus one warp/ block combine.  cnt16[w][b]
  // becomes the tile slot of warp w's first element of bucket b (the
  // bucket's tile offset plus the counts of the warps before w; < kTile, so
  // it fits 16 bits), which leaves the re-layout one lookup per element.
  int32_t my_total = 0;
  for (int b = b_lo; b < b_hi; ++b) {
    int32_t tot = 0;
#pragma unroll 4
    for (int ww = 0; ww < C::kWarps; ++ww) tot += cnt16[ww * buckets + b];
    toff[b] = tot;  // tile count for now
    my_total += tot + ((bulk && tot) ? 3 : 0);  // spare slots to align the run
  }
  // Block exclusive scan of my_total.
  __shared__ int32_t s_wsum[32];
  int32_t incl = my_total;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) s_wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    const int32_t x = lane < C::kWarps ? s_wsum[lane] : 0;
    int32_t xi = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, xi, d);
      if (lane >= d) xi += y;
    }
    if (lane < C::kWarps) s_wsum[lane] = xi - x;
  }
  __syncthreads();
  int32_t run = s_wsum[w] + (incl - my_total);
  auto warp_slots = [&](int b, int32_t start) {
#pragma unroll 4
    for (int ww = 0; ww < C::kWarps; ++ww) {
      const int32_t c = cnt16[ww * buckets + b];
      cnt16[ww * buckets + b] = static_cast<uint16_t>(start);
      start += c;
    }
  };
  // With `bulk`, the run's staging start takes the residue mod 4 of its
  // output start (within its 3 spare slots); each thread keeps its runs
  // (output start, staging start, count) for the bulk copies below.
  constexpr int kMaxOwn = 2;  // buckets per thread: 512 threads, up to 1024 buckets
  int32_t run_dst[kMaxOwn] = {0, 0}, run_src[kMaxOwn] = {0, 0}, run_cnt[kMaxOwn] = {0, 0};
  auto place = [&](int k, int b, int32_t dst) {
    const int32_t c = toff[b];
    const int32_t s = bulk ? run + static_cast<int32_t>((static_cast<uint32_t>(dst) -
                                                           static_cast<uint32_t>(run)) & 3u)
                           : run;
    // First output index of bucket b from this tile, minus its tile slot.
    gofs[b] = dst - s;
    warp_slots(b, s);
    if (k < kMaxOwn) {
      run_dst[k] = dst;
      run_src[k] = s;
      run_cnt[k] = c;
    }
    run += c + ((bulk && c) ? 3 : 0);
  };
#pragma unroll
  for (int k = 0; k < kHisPre; ++k) {
    const int b = b_lo + k;
    if (b < b_hi) place(k, b, his_pre[k]);
  }
  for (int b = b_lo + kHisPre; b < b_hi; ++b)
    place(b - b_lo, b, his[static_cast<int64_t>(b) * tiles + t]);
  __syncthreads();

  // -- two buckets: each warp's lanes of one bucket hold consecutive output
  // slots, so every store instruction covers at most two contiguous
  // stretches; write from registers, skipping the shared-memory re-layout
  // (2^28 pairs: 1.21 -> 1.11 ms; at 4 buckets even, at 8 and more slower,
  // the stores' sectors being only partly filled) --
  if (!kWide && buckets <= kDirectBuckets) {
#pragma unroll
    for (int it = 0; it < C::kIters; ++it) {
      const int pos = w * C::kSeg + it * 32 + lane;
      if (pos < count) {
        const int b = static_cast<int>((static_cast<unsigned>(kk[it]) >> shift) & mask);
        const int r = static_cast<int>((rk[it >> 1] >> ((it & 1) * 16)) & 0xffffu);
        const int64_t o = static_cast<int64_t>(gofs[b]) + cnt16[w * buckets + b] + r;
        if (LAYOUT == EDPP_KVS_AOS) {
          reinterpret_cast<int2 *>(keys_out)[o] = make_int2(kk[it], vv[it]);
        } else {
          keys_out[o] = kk[it];
          if (LAYOUT == EDPP_KVS_SOA) vals_out[o] = vv[it];
        }
      }
    }
    return;
  }

  // -- re-lay the tile out in bucket order (stable); without bulk copies the
  // key/value pairs of KVS_SOA are staged interleaved, one 8-byte store per
  // element (2^28 pairs: 32 to 1024 buckets 2-6% faster than two 4-byte
  // stores into separate arrays) --
#pragma unroll
  for (int it = 0; it < C::kIters; ++it) {
    const int pos = w * C::kSeg + it * 32 + lane;
    if (pos < count) {
      const int b = static_cast<int>((static_cast<unsigned>(kk[it]) >> shift) & mask);
      const int r = static_cast<int>((rk[it >> 1] >> ((it & 1) * 16)) & 0xffffu);
      const int s = cnt16[w * buckets + b] + r;
      if (LAYOUT == EDPP_KVS_AOS || (LAYOUT == EDPP_KVS_SOA && !bulk)) {
        s_pairs[s] = make_int2(kk[it], vv[it]);
      } else {
        s_keys[s] = kk[it];
        if (LAYOUT == EDPP_KVS_SOA) s_vals[s] = vv[it];
      }
    }
  }
  if (!kWide && bulk) {
    // -- write out: per bucket run, plain stores for the ragged ends and one
    // bulk copy per array for the 16-byte-aligned middle --
    fence_proxy_async_smem();  // the re-layout's writes before the copies read them
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kMaxOwn; ++k) {
      const int32_t c = run_cnt[k];
      if (k >= b_hi - b_lo || c == 0) continue;
      const int32_t d = run_dst[k], s = run_src[k];
      const int32_t head = min(c, static_cast<int32_t>((4u - (static_cast<uint32_t>(d) & 3u)) & 3u));
      const int32_t body = (c - head) & ~3;
      for (int i = 0; i < head; ++i) {
        keys_out[d + i] = s_keys[s + i];
        if (LAYOUT == EDPP_KVS_SOA) vals_out[d + i] = s_vals[s + i];
      }
      if (body) {
        tma_store_1d(keys_out + d + head, s_keys + s + head, static_cast<uint32_t>(body) * 4u);
        if (LAYOUT == EDPP_KVS_SOA)
          tma_store_1d(vals_out + d + head, s_vals + s + head, static_cast<uint32_t>(body) * 4u);
      }
      for (int i = head + body; i < c; ++i) {
        keys_out[d + i] = s_keys[s + i];
        if (LAYOUT == EDPP_KVS_SOA) vals_out[d + i] = s_vals[s + i];
      }
    }
    tma_store_commit();
    tma_store_wait_all();  // the copies are complete before the block's shared memory goes
    return;
  }
  __syncthreads();

  // -- write out: consecutive threads write consecutive slots of a bucket run --
  for (int s = tid; s < count; s += THREADS) {
    if (LAYOUT == EDPP_KVS_AOS) {
      const int2 p = s_pairs[s];
      const int b = static_cast<int>((static_cast<unsigned>(p.x) >> shift) & mask);
      reinterpret_cast<int2 *>(keys_out)[gofs[b] + s] = p;
    } else if (LAYOUT == EDPP_KVS_SOA) {
      const int2 p = s_pairs[s];
      const int b = static_cast<int>((static_cast<unsigned>(p.x) >> shift) & mask);
      const int64_t o = static_cast<int64_t>(gofs[b]) + s;
      keys_out[o] = p.x;
      vals_out[o] = p.y;
    } else {
      const int32_t key = s_keys[s];
      const int b = static_cast<int>((static_cast<unsigned>(key) >> shift) & mask);
      const int64_t o = static_cast<int64_t>(gofs[b]) + s;
      keys_out[o] = key;
      if (LAYOUT == EDPP_KVS_SOA) vals_out[o] = s_vals[s];
    }
  }
}

// bucket_start[b] = his[b*T] (gatherStartPos, split_kernel.cl:320-332).
__global__ void bucket_start_kernel(const int32_t *his, int64_t tiles, int buckets,
                                    int32_t *start) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < buckets; b += gridDim.x * blockDim.x)
    start[b] = his[static_cast<int64_t>(b) * tiles];
}

size_t his_bytes(int64_t tiles, int buckets) {
  return round_up(static_cast<size_t>(tiles) * buckets * 4, 256);
}

template <int THREADS, int LAYOUT, bool kWide> int set_smem_attr() {
  static std::once_flag once[64];
  static int status[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::call_once(once[dev], [&] {
    const size_t bytes = scatter_smem_bytes<THREADS, LAYOUT>(kWide ? kOnePassMax : 256, true);
    status[dev] = cuda_status(cudaFuncSetAttribute(split_scatter_kernel<THREADS, LAYOUT, kWide>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   static_cast<int>(bytes)));
  });
  return status[dev];
}

template <int THREADS, int LAYOUT>
int launch_scatter(const int32_t *keys_in, int32_t *keys_out, const int32_t *vals_in,
                   int32_t *vals_out, int64_t n, int buckets, int shift, int64_t tiles,
                   const int32_t *his, bool tma, cudaStream_t st) {
  const bool wide = buckets > 256;
  const int s = wide ? set_smem_attr<THREADS, LAYOUT, true>() : set_smem_attr<THREADS, LAYOUT, false>();
  if (s != EDPP_OK) return s;
  const bool bulk = LAYOUT != EDPP_KVS_AOS && buckets > kDirectBuckets &&
                    buckets <= kBulkBuckets && aligned16(keys_out) &&
                    (LAYOUT != EDPP_KVS_SOA || aligned16(vals_out));
  const size_t smem = scatter_smem_bytes<THREADS, LAYOUT>(buckets, bulk);
  const unsigned grid = static_cast<unsigned>(tiles);
  if (wide)
    split_scatter_kernel<THREADS, LAYOUT, true><<<grid, THREADS, smem, st>>>(
        keys_in, keys_out, vals_in, vals_out, n, buckets, shift, tiles, his, tma, bulk,
        kDefaultWaitNs, fault_word());
  else
    split_scatter_kernel<THREADS, LAYOUT, false><<<grid, THREADS, smem, st>>>(
        keys_in, keys_out, vals_in, vals_out, n, buckets, shift, tiles, his, tma, bulk,
        kDefaultWaitNs, fault_word());
  return launch_status();
}

template <int LAYOUT>
int split_layout(const int32_t *keys_in, int32_t *keys_out, int32_t *bucket_start, int64_t n,
                 int buckets, const int32_t *vals_in, int32_t *vals_out, void *ws, size_t ws_bytes,
                 cudaStream_t st, int shift = 0) {
  if (buckets > kOnePassMax) return EDPP_EINVAL;  // callers take two passes from 2048 on
  const int64_t tiles = (n + kTile - 1) / kTile;
  int32_t *his = static_cast<int32_t *>(ws);
  const int64_t hlen = tiles * buckets;
  void *scan_ws = static_cast<char *>(ws) + his_bytes(tiles, buckets);
  const size_t scan_ws_bytes = ws_bytes - his_bytes(tiles, buckets);
  bool tma = aligned16(keys_in) && (LAYOUT != EDPP_KVS_SOA || aligned16(vals_in));
  split_hist_kernel<LAYOUT><<<static_cast<unsigned>(tiles), kHistThreads, 0, st>>>(
      keys_in, n, buckets, shift, tiles, his, aligned16(keys_in));
  int s = launch_status();
  if (s != EDPP_OK) return s;
  s = edpp_scan_exclusive_i32(his, his, hlen, EDPP_SCAN_LOOKBACK, scan_ws, scan_ws_bytes, st);
  if (s != EDPP_OK) return s;
  if (bucket_start) {
    bucket_start_kernel<<<(buckets + 255) / 256, 256, 0, st>>>(his, tiles, buckets, bucket_start);
    s = launch_status();
    if (s != EDPP_OK) return s;
  }
  return launch_scatter<512, LAYOUT>(keys_in, keys_out, vals_in, vals_out, n, buckets, shift,
                                     tiles, his, tma, st);
}

// From kLsdBuckets buckets on, a split is two stable passes through a
// temporary copy: by the low 8 bits of the bucket, then by the rest (the
// output is ordered by (high, low) bits, ties in input order: the same stable
// split).  One pass ranks with 11-12 bits per element and stays below a third
// of the two passes' speed (B = 4096 at 2^26 keys: 1.57 ms one pass).
constexpr int kLsdBuckets = 2048;

size_t split_pass_ws_bytes(int64_t n, int buckets) {
  const int64_t tiles = (n + kTile - 1) / kTile;
  return his_bytes(tiles, buckets) +
         edpp_scan_workspace_size(tiles * buckets, EDPP_I32, EDPP_SCAN_LOOKBACK);
}

// LSD workspace: temporary keys and values (two arrays of 4 bytes per
// element, or {key,value} pairs over both), the bucket totals, then the
// passes' workspace.
size_t lsd_half_bytes(int64_t n) { return round_up(static_cast<size_t>(n) * 4, 256); }
size_t lsd_tmp_bytes(int64_t n) { return 2 * lsd_half_bytes(n); }

size_t split_ws_bytes(int64_t n, int buckets) {
  if (n <= 0 || buckets < 1) return 0;
  if (buckets >= kLsdBuckets)
    return lsd_tmp_bytes(n) + round_up(static_cast<size_t>(buckets) * 4, 256) +
           std::max(split_pass_ws_bytes(n, 256), split_pass_ws_bytes(n, buckets >> 8));
  return split_pass_ws_bytes(n, buckets);
}

// Bucket totals of the keys (bucket = key & (B-1)), for the bucket starts of
// a two-pass split.  totals[] zeroed by the caller.
template <int LAYOUT>
__global__ void __launch_bounds__(kHistThreads)
    bucket_totals_kernel(const int32_t *__restrict__ keys, int64_t n, int buckets,
                         int32_t *__restrict__ totals) {
  __shared__ uint32_t cnt[kMaxBuckets];
  const unsigned mask = static_cast<unsigned>(buckets - 1);
  for (int b = threadIdx.x; b < buckets; b += kHistThreads) cnt[b] = 0;
  __syncthreads();
  const int64_t stride = static_cast<int64_t>(gridDim.x) * kHistThreads;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * kHistThreads + threadIdx.x; i < n; i += stride)
    atomicAdd(&cnt[static_cast<unsigned>(key_at<LAYOUT>(keys, i)) & mask], 1u);
  __syncthreads();
  for (int b = threadIdx.x; b < buckets; b += kHistThreads)
    if (cnt[b]) atomicAdd(reinterpret_cast<unsigned *>(totals + b), cnt[b]);
}

// start[b] = sum of totals[0..b), one block.
__global__ void __launch_bounds__(1024)
    bucket_start_from_totals_kernel(const int32_t *__restrict__ totals, int buckets,
                                    int32_t *__restrict__ start) {
  __shared__ int32_t wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (buckets + 1023) / 1024;
  const int lo = min(buckets, t * per), hi = min(buckets, lo + per);
  int32_t s = 0;
  for (int b = lo; b < hi; ++b) s += totals[b];
  int32_t incl = s;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    const int32_t x = wsum[lane];
    int32_t xi = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, xi, d);
      if (lane >= d) xi += y;
    }
    wsum[lane] = xi - x;
  }
  __syncthreads();
  int32_t run = wsum[w] + incl - s;
  for (int b = lo; b < hi; ++b) {
    start[b] = run;
    run += totals[b];
  }
}

template <int LAYOUT>
int split_lsd(const int32_t *keys_in, int32_t *keys_out, int32_t *bucket_start, int64_t n,
              int buckets, const int32_t *vals_in, int32_t *vals_out, void *ws, size_t ws_bytes,
              cudaStream_t st) {
  char *w = static_cast<char *>(ws);
  const size_t tmp = lsd_tmp_bytes(n);
  int32_t *tk = reinterpret_cast<int32_t *>(w);  // keys, or {key,value} pairs
  int32_t *tv = LAYOUT == EDPP_KVS_SOA ? reinterpret_cast<int32_t *>(w + lsd_half_bytes(n)) : nullptr;
  int32_t *totals = reinterpret_cast<int32_t *>(w + tmp);
  const size_t used = tmp + round_up(static_cast<size_t>(buckets) * 4, 256);
  void *pws = w + used;
  const size_t pws_bytes = ws_bytes - used;
  int s = split_layout<LAYOUT>(keys_in, tk, nullptr, n, 256, vals_in, tv, pws, pws_bytes, st, 0);
  if (s != EDPP_OK) return s;
  s = split_layout<LAYOUT>(tk, keys_out, nullptr, n, buckets >> 8, tv, vals_out, pws, pws_bytes,
                           st, 8);
  if (s != EDPP_OK || !bucket_start) return s;
  if (cudaMemsetAsync(totals, 0, static_cast<size_t>(buckets) * 4, st) != cudaSuccess)
    return EDPP_ECUDA;
  const int64_t blocks = min64(static_cast<int64_t>(device_sm_count()) * 4,
                               (n + kHistThreads - 1) / kHistThreads);
  // the output holds the same keys (and is valid when it aliases the input)
  bucket_totals_kernel<LAYOUT><<<static_cast<unsigned>(max64(blocks, 1)), kHistThreads, 0, st>>>(
      keys_out, n, buckets, totals);
  bucket_start_from_totals_kernel<<<1, 1024, 0, st>>>(totals, buckets, bucket_start);
  return launch_status();
}

}  // namespace
}  // namespace edpp

extern "C" {

size_t edpp_split_workspace_size(int64_t length, int buckets, int layout) {
  (void)layout;
  if (buckets < 1 || buckets > edpp::kMaxBuckets || (buckets & (buckets - 1))) return 0;
  return edpp::split_ws_bytes(length, buckets);
}

int edpp_split_i32(const int32_t *keys_in, int32_t *keys_out, int32_t *bucket_start,
                   int64_t length, int buckets, int layout, const int32_t *vals_in,
                   int32_t *vals_out, void *ws, size_t ws_bytes, void *stream) {
  if (length < 0 || length > INT32_MAX) return EDPP_EINVAL;
  if (buckets < 1 || buckets > edpp::kMaxBuckets || (buckets & (buckets - 1))) return EDPP_EINVAL;
  if (layout != EDPP_KO && layout != EDPP_KVS_AOS && layout != EDPP_KVS_SOA) return EDPP_EINVAL;
  if (length == 0) return EDPP_OK;
  if (!keys_in || !keys_out) return EDPP_EINVAL;
  // SOA needs both value arrays (splitImpl.cpp:29-34 returns -1 otherwise).
  if (layout == EDPP_KVS_SOA && (!vals_in || !vals_out)) return EDPP_EINVAL;
  const size_t need = edpp::split_ws_bytes(length, buckets);
  if (!ws || ws_bytes < need) return EDPP_ENOMEM;
  cudaStream_t st = edpp::as_stream(stream);
  if (buckets >= edpp::kLsdBuckets) {
    switch (layout) {
      case EDPP_KO:
        return edpp::split_lsd<EDPP_KO>(keys_in, keys_out, bucket_start, length, buckets, nullptr,
                                        nullptr, ws, ws_bytes, st);
      case EDPP_KVS_SOA:
        return edpp::split_lsd<EDPP_KVS_SOA>(keys_in, keys_out, bucket_start, length, buckets,
                                             vals_in, vals_out, ws, ws_bytes, st);
      default:
        return edpp::split_lsd<EDPP_KVS_AOS>(keys_in, keys_out, bucket_start, length, buckets,
                                             nullptr, nullptr, ws, ws_bytes, st);
    }
  }
  switch (layout) {
    case EDPP_KO:
      return edpp::split_layout<EDPP_KO>(keys_in, keys_out, bucket_start, length, buckets, nullptr,
                                         nullptr, ws, ws_bytes, st);
    case EDPP_KVS_SOA:
      return edpp::split_layout<EDPP_KVS_SOA>(keys_in, keys_out, bucket_start, length, buckets,
                                              vals_in, vals_out, ws, ws_bytes, st);
    default:
      return edpp::split_layout<EDPP_KVS_AOS>(keys_in, keys_out, bucket_start, length, buckets,
                                              nullptr, nullptr, ws, ws_bytes, st);
  }
}

}  // extern "C"

// ---- LSD radix sort on the stable split -----------------------------------------
// Sorts (key, value) pairs by the key's bit pattern (unsigned order) over bits
// [begin_bit, end_bit), 8 bits per pass, each pass one stable split by the
// digit (key >> shift) & 255, ping-ponging through the workspace; the last
// pass lands in the caller's output.  Follows the reference's LSD radix sort
// (obsolete/CUDA/kernels/radixSort.cu:333-357: histogram, scan, scatter per
// digit over all bits of the key), with the GB300 split as the per-digit pass.
namespace {

size_t radix_ws_bytes(int64_t n, bool with_values) {
  const size_t buf = edpp::round_up(static_cast<size_t>(n) * 4, 256);
  return buf * (with_values ? 2 : 1) + edpp::split_ws_bytes(n, 256);
}

}  // namespace

extern "C" size_t edpp_radix_sort_workspace_size(int64_t length, int with_values) {
  if (length <= 0) return 0;
  return radix_ws_bytes(length, with_values != 0);
}

extern "C" int edpp_radix_sort_i32(const int32_t *keys_in, int32_t *keys_out,
                                   const int32_t *vals_in, int32_t *vals_out, int64_t length,
                                   int begin_bit, int end_bit, void *ws, size_t ws_bytes,
                                   void *stream) {
  using namespace edpp;
  if (length < 0 || length > INT32_MAX) return EDPP_EINVAL;
  if (begin_bit < 0 || end_bit > 32 || begin_bit > end_bit) return EDPP_EINVAL;
  const bool kv = vals_in != nullptr;
  if (kv && !vals_out) return EDPP_EINVAL;
  if (length == 0) return EDPP_OK;
  if (!keys_in || !keys_out || keys_in == keys_out || (kv && vals_in == vals_out))
    return EDPP_EINVAL;
  if (!ws || ws_bytes < radix_ws_bytes(length, kv)) return EDPP_ENOMEM;
  cudaStream_t st = as_stream(stream);
  const size_t bytes = static_cast<size_t>(length) * 4;
  if (begin_bit == end_bit) {  // no digit: a copy
    if (cudaMemcpyAsync(keys_out, keys_in, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return EDPP_ECUDA;
    if (kv && cudaMemcpyAsync(vals_out, vals_in, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return EDPP_ECUDA;
    return EDPP_OK;
  }
  const size_t buf = round_up(bytes, 256);
  char *w = static_cast<char *>(ws);
  int32_t *tk = reinterpret_cast<int32_t *>(w);
  int32_t *tv = kv ? reinterpret_cast<int32_t *>(w + buf) : nullptr;
  void *sws = w + buf * (kv ? 2 : 1);
  const size_t sws_bytes = ws_bytes - buf * (kv ? 2 : 1);
  const int passes = (end_bit - begin_bit + 7) / 8;
  const int32_t *sk = keys_in, *sv = vals_in;
  for (int i = 0; i < passes; ++i) {
    const int shift = begin_bit + 8 * i;
    const int bits = std::min(8, end_bit - shift);
    const bool to_out = ((passes - 1 - i) % 2) == 0;
    int32_t *dk = to_out ? keys_out : tk;
    int32_t *dv = kv ? (to_out ? vals_out : tv) : nullptr;
    const int s = kv ? split_layout<EDPP_KVS_SOA>(sk, dk, nullptr, length, 1 << bits, sv, dv, sws,
                                                  sws_bytes, st, shift)
                     : split_layout<EDPP_KO>(sk, dk, nullptr, length, 1 << bits, nullptr, nullptr,
                                             sws, sws_bytes, st, shift);
    if (s != EDPP_OK) return s;
    sk = dk;
    sv = dv;
  }
  return EDPP_OK;
}

// ---- WI_split order -----------------------------------------------------------------
// The reference's WI_split (opencl/kernels/split_kernel.cl:335-412, with
// compute_mixed_access, scan_global_RSS_kernel.cl:37-48) gives work-item
// g = chunk*step + lane the indices chunk*C + lane + step*k of its chunk
// (C = step*tile, step = min(local_size, 32), tile = ceil(n / (local_size *
// grid_size))) and writes them bucket-major, then by g, then by k.  That is
// the stable split of the input visited in (chunk, lane, k) order, so this
// mode gathers the input into that order and runs the stable split.  With
// tile == 1 (n <= local_size*grid_size) the order is the stable order.
namespace edpp {
namespace {

template <int LAYOUT>
__global__ void wi_permute_kernel(const int32_t *__restrict__ keys, const int32_t *__restrict__ vals,
                                  int32_t *__restrict__ tk, int32_t *__restrict__ tv, int64_t n,
                                  int64_t chunk, int64_t step) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; j < n; j += stride) {
    const int64_t c = j / chunk, r = j - c * chunk;
    const int64_t len = min64(chunk, n - c * chunk);
    const int64_t base = len / step, rem = len % step;
    int64_t lane, k;
    if (r < rem * (base + 1)) {
      lane = r / (base + 1);
      k = r - lane * (base + 1);
    } else {
      const int64_t r2 = r - rem * (base + 1);
      lane = rem + r2 / base;
      k = r2 - (lane - rem) * base;
    }
    const int64_t i = c * chunk + lane + step * k;
    if (LAYOUT == EDPP_KVS_AOS) {
      tk[2 * j] = keys[2 * i];
      tk[2 * j + 1] = keys[2 * i + 1];
    } else {
      tk[j] = keys[i];
      if (LAYOUT == EDPP_KVS_SOA) tv[j] = vals[i];
    }
  }
}

size_t wi_tmp_bytes(int64_t n, int layout) {
  const size_t one = round_up(static_cast<size_t>(n) * 4, 256);
  return layout == EDPP_KO ? one : 2 * one;
}

}  // namespace
}  // namespace edpp

extern "C" size_t edpp_split_wi_workspace_size(int64_t length, int buckets, int layout) {
  const size_t sw = edpp_split_workspace_size(length, buckets, layout);
  if (sw == 0) return 0;
  return edpp::wi_tmp_bytes(length, layout) + sw;
}

extern "C" int edpp_split_i32_wi(const int32_t *keys_in, int32_t *keys_out, int64_t length,
                                 int buckets, int layout, const int32_t *vals_in,
                                 int32_t *vals_out, int local_size, int grid_size, void *ws,
                                 size_t ws_bytes, void *stream) {
  using namespace edpp;
  if (local_size < 1 || grid_size < 1) return EDPP_EINVAL;
  if (length < 0 || length > INT32_MAX) return EDPP_EINVAL;
  if (buckets < 1 || buckets > kMaxBuckets || (buckets & (buckets - 1))) return EDPP_EINVAL;
  if (layout != EDPP_KO && layout != EDPP_KVS_AOS && layout != EDPP_KVS_SOA) return EDPP_EINVAL;
  if (length == 0) return EDPP_OK;
  if (!keys_in || !keys_out) return EDPP_EINVAL;
  if (layout == EDPP_KVS_SOA && (!vals_in || !vals_out)) return EDPP_EINVAL;
  const int64_t G = static_cast<int64_t>(local_size) * grid_size;
  const int64_t step = local_size < 32 ? local_size : 32;
  const int64_t tile = (length + G - 1) / G;
  const size_t tmp = wi_tmp_bytes(length, layout);
  if (!ws || ws_bytes < tmp + edpp_split_workspace_size(length, buckets, layout)) return EDPP_ENOMEM;
  if (tile == 1)
    return edpp_split_i32(keys_in, keys_out, nullptr, length, buckets, layout, vals_in, vals_out,
                          static_cast<char *>(ws) + tmp, ws_bytes - tmp, stream);
  cudaStream_t st = as_stream(stream);
  int32_t *tk = static_cast<int32_t *>(ws);
  int32_t *tv = layout == EDPP_KVS_SOA
                    ? reinterpret_cast<int32_t *>(static_cast<char *>(ws) + tmp / 2)
                    : nullptr;
  const unsigned blocks = static_cast<unsigned>(min64((length + 255) / 256, device_sm_count() * 8));
  if (layout == EDPP_KO)
    wi_permute_kernel<EDPP_KO><<<blocks, 256, 0, st>>>(keys_in, nullptr, tk, nullptr, length,
                                                        step * tile, step);
  else if (layout == EDPP_KVS_SOA)
    wi_permute_kernel<EDPP_KVS_SOA><<<blocks, 256, 0, st>>>(keys_in, vals_in, tk, tv, length,
                                                             step * tile, step);
  else
    wi_permute_kernel<EDPP_KVS_AOS><<<blocks, 256, 0, st>>>(keys_in, nullptr, tk, nullptr, length,
                                                             step * tile, step);
  const int s = launch_status();
  if (s != EDPP_OK) return s;
  return edpp_split_i32(tk, keys_out, nullptr, length, buckets, layout, tv, vals_out,
                        static_cast<char *>(ws) + tmp, ws_bytes - tmp, stream);
}
