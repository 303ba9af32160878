// gather_scatter_part.cu — partitioned multi-pass gather and scatter.
//
// Same results as the windowed passes of gather_scatter.cu (and of the
// reference's gatherImpl.cpp:38-53 / scatterImpl.cpp:39-52), scheduled for
// GB300's memory system.  On a random permutation of 2^28 int32 the direct
// passes are bound by DRAM random access: every missed 4-byte load pulls
// 64-128 bytes from DRAM and every 4-byte store to a sector not in L2 costs a
// fill read plus a sector write.  Here the pass windows become partitions:
//
//   count      valid indices per window (P windows of W = 2^k elements)
//   bases      exclusive scan of the counts -> write cursor of each window
//   partition  each block stages a tile, groups its (index, payload) pairs
//              by window in shared memory and appends one contiguous run per
//              window at the window's cursor (coalesced 8-byte pairs)
//   scatter:   apply  — pairs are consumed in window order through an atomic
//              chunk ticket, so all SMs work inside one window at a time and
//              the random stores land in an L2-resident slice of out[]
//   gather:    fetch  — the same ordered sweep reads in[] inside an
//              L2-resident window and regroups (i, value) by destination
//              window (capacity W each: every i occurs once);
//              apply  — ordered sweep over destination windows, out[i] = v
//
// Traffic per element: scatter 32 B, gather 48 B, nearly all streaming,
// against 12 B algorithmic.  Indices outside [0,n) are dropped at `count`
// and `partition`, as every pass of the windowed form skips them.  Scatter
// with repeated destinations keeps one of the colliding values (unspecified
// which), as the reference's racing stores do.
#include <mutex>

#include "common.cuh"
#include "tune.h"

namespace edpp {
namespace {

constexpr int kThreads = 256;
constexpr int kPer = 16;                    // elements per thread per tile
constexpr int kTile = kThreads * kPer;      // 4096
constexpr int kMaxWin = 2048;               // windows
constexpr int64_t kMinWin = 1024;           // elements per window, at least
constexpr int kChunk = 8192;                // pairs per ticket in ordered sweeps
constexpr size_t kHdr = 256;                // tickets

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Random read of a payload element: a plain global load (the read-only
// .nc path measured much slower for random 4-byte reads on GB300).
__device__ __forceinline__ int ld_random(const int32_t *p) { return *p; }

// A slot for this lane's element among the tile's elements of window w (-1:
// invalid): one shared-memory atomic per element.  Slots within a window come
// in no particular order, which no caller depends on.  (Grouping lanes with
// __match_any_sync first costs several times more: on this GPU the match
// instruction, not memory, bounded these kernels.)
__device__ __forceinline__ int rank_in_window(int w, uint32_t *scnt, unsigned) {
  return w >= 0 ? static_cast<int>(atomicAdd(&scnt[w], 1u)) : -1;
}

// Block-wide exclusive scan of scnt[0..nwin) into soff[], returns total.
// NT threads in the block; s_warp holds NT/32 + 1 entries.
template <int NT = kThreads>
__device__ __forceinline__ uint32_t block_scan_counts(const uint32_t *scnt, uint32_t *soff, int nwin,
                                                      uint32_t *s_warp) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int per = (nwin + NT - 1) / NT;
  const int lo = min(nwin, tid * per), hi = min(nwin, lo + per);
  uint32_t s = 0;
  for (int i = lo; i < hi; ++i) s += scnt[i];
  uint32_t incl = s;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) s_warp[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    const uint32_t x = lane < NT / 32 ? s_warp[lane] : 0u;
    uint32_t xi = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, xi, d);
      if (lane >= d) xi += y;
    }
    if (lane < NT / 32) s_warp[lane] = xi - x;
    if (lane == 31) s_warp[NT / 32] = xi;  // total
  }
  __syncthreads();
  uint32_t run = s_warp[wid] + (incl - s);
  for (int i = lo; i < hi; ++i) {
    soff[i] = run;
    run += scnt[i];
  }
  const uint32_t total = s_warp[NT / 32];
  __syncthreads();
  return total;
}

// ---- count ----------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
    part_count_kernel(const int32_t *__restrict__ loc, int64_t n, int log_w, int nwin,
                      uint32_t *__restrict__ cnt, bool vec) {
  extern __shared__ uint32_t scnt[];
  for (int i = threadIdx.x; i < nwin; i += kThreads) scnt[i] = 0;
  __syncthreads();
  const unsigned lt = lanemask_lt();
  const int64_t stride = static_cast<int64_t>(gridDim.x) * kThreads;
  auto one = [&](int32_t l, bool in_range) {
    const bool valid = in_range && static_cast<uint64_t>(static_cast<uint32_t>(l)) <
                                       static_cast<uint64_t>(n) && l >= 0;
    rank_in_window(valid ? (l >> log_w) : -1, scnt, lt);
  };
  if (vec) {
    const int64_t n4 = n >> 2;
    const int4 *l4 = reinterpret_cast<const int4 *>(loc);
    const int64_t base0 = static_cast<int64_t>(blockIdx.x) * kThreads;
    for (int64_t b = base0; b < n4; b += stride) {
      const int64_t i = b + threadIdx.x;
      int4 q = make_int4(-1, -1, -1, -1);
      const bool ok = i < n4;
      if (ok) q = __ldcs(l4 + i);
      one(q.x, ok);
      one(q.y, ok);
      one(q.z, ok);
      one(q.w, ok);
    }
    // tail
    if (blockIdx.x == 0) {
      const int64_t i = 4 * n4 + threadIdx.x;
      const bool ok = threadIdx.x < 32 && i < n;
      if (threadIdx.x < 32) one(ok ? loc[i] : -1, ok);
    }
  } else {
    const int64_t base0 = static_cast<int64_t>(blockIdx.x) * kThreads;
    for (int64_t b = base0; b < n; b += stride) {
      const int64_t i = b + threadIdx.x;
      const bool ok = i < n;
      one(ok ? loc[i] : -1, ok);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nwin; i += kThreads)
    if (scnt[i]) atomicAdd(&cnt[i], scnt[i]);
}

// ---- bases: fill[w] = sum of cnt[0..w); fill2[w] = w * W (gather) ------------------
__global__ void __launch_bounds__(kThreads)
    part_bases_kernel(const uint32_t *cnt, uint32_t *fill, uint32_t *fill2, int nwin, int64_t w_elems,
                      uint32_t *total) {
  __shared__ uint32_t scnt[kMaxWin], soff[kMaxWin], s_warp[16];
  for (int i = threadIdx.x; i < nwin; i += kThreads) scnt[i] = cnt[i];
  __syncthreads();
  const uint32_t t = block_scan_counts(scnt, soff, nwin, s_warp);
  for (int i = threadIdx.x; i < nwin; i += kThreads) {
    fill[i] = soff[i];
    if (fill2) fill2[i] = static_cast<uint32_t>(static_cast<int64_t>(i) * w_elems);
  }
  if (threadIdx.x == 0) *total = t;
}

// Group the block's pairs by window and append one run per window at the
// window's global cursor.  pair.x determines the window (x >> log_w); w[e] is
// -1 for dropped elements; rank[e] from rank_in_window.
template <int PER, int NT = kThreads>
__device__ __forceinline__ void flush_runs(const int2 (&pr)[PER], const int (&w)[PER],
                                           const int (&rank)[PER], int nwin, int log_w,
                                           uint32_t *scnt, uint32_t *soff, uint32_t *sgb,
                                           uint32_t *s_warp, int2 *stage, uint32_t *fill,
                                           int2 *__restrict__ dst) {
  const uint32_t total = block_scan_counts<NT>(scnt, soff, nwin, s_warp);
  // sgb[w]: global index of the window's run minus its staging offset
  // (modulo 2^32), so a staged slot s maps to dst[sgb[w] + s].  The first
  // claim of each thread is consumed only after the staging writes, so its
  // round trip to L2 overlaps them.
  const int i0 = threadIdx.x;
  const uint32_t c0 = i0 < nwin ? scnt[i0] : 0u;
  const uint32_t g0 = c0 ? atomicAdd(&fill[i0], c0) : 0u;
  for (int i = i0 + NT; i < nwin; i += NT)
    if (scnt[i]) sgb[i] = atomicAdd(&fill[i], scnt[i]) - soff[i];
#pragma unroll
  for (int e = 0; e < PER; ++e)
    if (w[e] >= 0) stage[soff[w[e]] + rank[e]] = pr[e];
  if (c0) sgb[i0] = g0 - soff[i0];
  __syncthreads();
  for (uint32_t s = threadIdx.x; s < total; s += NT) {
    const int2 p = stage[s];
    dst[sgb[p.x >> log_w] + s] = p;
  }
}

// The pipelined stages (partition, refine, fetch) group a tile with four
// barriers: (A) rank atomics done; claim_runs; (B) staging offsets known;
// staging writes and publish_run_bases; (C) runs staged; read-out.
//
// claim_runs, between A and B: thread t owns windows [t*per, t*per + per),
// per = ceil(nwin / NT) <= MAXPER.  For each owned window with pairs it
// claims the tile's run at the window's global cursor (g), resets the
// counter for the next tile, and sets the window's staging offset (o, and
// soff[] for the staging writes).  Warps take their part of the staging area
// in arrival order, by one shared atomic on *s_total (zero on entry; the
// tile's pair count after B): windows need disjoint contiguous ranges, not
// ordered ones.  The claims are consumed only by publish_run_bases, after
// the staging writes, so their round trip to L2 overlaps both.
template <int MAXPER, int NT>
__device__ __forceinline__ void claim_runs(uint32_t *scnt, uint32_t *soff, int nwin,
                                           uint32_t *__restrict__ fill, uint32_t *s_total,
                                           uint32_t (&g)[MAXPER], uint32_t (&o)[MAXPER]) {
  const int lane = threadIdx.x & 31;
  const int per = (nwin + NT - 1) / NT;
  const int lo = static_cast<int>(threadIdx.x) * per;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < MAXPER; ++k) {
    const int i = lo + k;
    const uint32_t c = (k < per && i < nwin) ? scnt[i] : 0u;
    g[k] = c ? atomicAdd(&fill[i], c) : 0u;
    if (c) scnt[i] = 0u;
    o[k] = s;
    s += c;
  }
  uint32_t incl = s;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  uint32_t wb = 0;
  if (lane == 31 && incl) wb = atomicAdd(s_total, incl);
  const uint32_t base = __shfl_sync(0xffffffffu, wb, 31) + incl - s;
#pragma unroll
  for (int k = 0; k < MAXPER; ++k) {
    o[k] += base;
    if (k < per && lo + k < nwin) soff[lo + k] = o[k];
  }
}

// sgb[w] = global index of window w's run minus its staging offset (modulo
// 2^32), so a staged slot s maps to dst[sgb[w] + s].
template <int MAXPER, int NT>
__device__ __forceinline__ void publish_run_bases(uint32_t *sgb, int nwin, const uint32_t (&g)[MAXPER],
                                                  const uint32_t (&o)[MAXPER]) {
  const int per = (nwin + NT - 1) / NT;
  const int lo = static_cast<int>(threadIdx.x) * per;
#pragma unroll
  for (int k = 0; k < MAXPER; ++k)
    if (k < per && lo + k < nwin) sgb[lo + k] = g[k] - o[k];
}

// ---- partition -------------------------------------------------------------------
// Gather pairs {loc, i}; scatter pairs {loc, in[i]}.
template <bool kScatter>
__global__ void __launch_bounds__(kThreads)
    part_partition_kernel(const int32_t *__restrict__ loc, const int32_t *__restrict__ in, int64_t n,
                          int log_w, int nwin, uint32_t *__restrict__ fill, int2 *__restrict__ pairs,
                          bool vec) {
  extern __shared__ __align__(16) unsigned char smem[];
  int2 *stage = reinterpret_cast<int2 *>(smem);
  uint32_t *scnt = reinterpret_cast<uint32_t *>(stage + kTile);
  uint32_t *soff = scnt + nwin;
  uint32_t *sgb = soff + nwin;
  __shared__ uint32_t s_warp[16];
  for (int i = threadIdx.x; i < nwin; i += kThreads) scnt[i] = 0;
  __syncthreads();
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kTile;
  const int t = threadIdx.x;
  const unsigned lt = lanemask_lt();
  int2 pr[kPer];
  int w[kPer], rank[kPer];
#pragma unroll
  for (int k = 0; k < kPer / 4; ++k) {
    const int64_t i0 = base + static_cast<int64_t>(k * kThreads + t) * 4;  // 4 elements
    int4 l = make_int4(-1, -1, -1, -1), v = make_int4(0, 0, 0, 0);
    if (vec && i0 + 3 < n) {
      l = __ldcs(reinterpret_cast<const int4 *>(loc + i0));
      if (kScatter) v = __ldcs(reinterpret_cast<const int4 *>(in + i0));
    } else {
      if (i0 + 0 < n) { l.x = loc[i0 + 0]; if (kScatter) v.x = in[i0 + 0]; }
      if (i0 + 1 < n) { l.y = loc[i0 + 1]; if (kScatter) v.y = in[i0 + 1]; }
      if (i0 + 2 < n) { l.z = loc[i0 + 2]; if (kScatter) v.z = in[i0 + 2]; }
      if (i0 + 3 < n) { l.w = loc[i0 + 3]; if (kScatter) v.w = in[i0 + 3]; }
    }
    const int32_t ls[4] = {l.x, l.y, l.z, l.w};
    const int32_t vs[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = 4 * k + q;
      const bool valid = (i0 + q < n) && ls[q] >= 0 && static_cast<int64_t>(ls[q]) < n;
      w[e] = valid ? (ls[q] >> log_w) : -1;
      pr[e] = make_int2(ls[q], kScatter ? vs[q] : static_cast<int32_t>(i0 + q));
      rank[e] = rank_in_window(w[e], scnt, lt);
    }
  }
  __syncthreads();
  flush_runs<kPer>(pr, w, rank, nwin, log_w, scnt, soff, sgb, s_warp, stage, fill, pairs);
}

// Pipelined form of the partition for 16-byte-aligned loc (and in): persistent
// blocks take tiles blockIdx, +gridDim, ...; the tile after next is copied
// into shared memory by TMA (loc, and in for a scatter, on one barrier) while
// the current one is grouped; the landed buffer then serves as the staging
// area of the runs.  Elements past the bulk copy (a ragged last tile) are read
// from global memory by the thread that ranks them.  nwin <= MAXPER * kThreads.
// Same output as part_partition_kernel.
template <bool kScatter, int MAXPER>
__global__ void __launch_bounds__(kThreads, MAXPER == 1 ? 3 : 2)
    part_partition_pipe_kernel(const int32_t *__restrict__ loc, const int32_t *__restrict__ in,
                               int64_t n, int log_w, int nwin, uint32_t *__restrict__ fill,
                               int2 *__restrict__ pairs, uint64_t timeout_ns, unsigned *fault) {
  extern __shared__ __align__(16) unsigned char smem[];
  int32_t *bufs = reinterpret_cast<int32_t *>(smem);  // [2][2 * kTile]: loc | in
  uint32_t *scnt = reinterpret_cast<uint32_t *>(bufs + 4 * kTile);
  uint32_t *soff = scnt + nwin;
  uint32_t *sgb = soff + nwin;
  __shared__ alignas(8) uint64_t bar[2];
  __shared__ uint32_t s_total;
  const int t = threadIdx.x;
  const int64_t G = gridDim.x;
  const int64_t tiles = (n + kTile - 1) / kTile;
  // bytes of tile `tl` that go by bulk copy (per array); the rest by plain loads
  auto bulk_of = [&](int64_t tl) {
    return static_cast<uint32_t>(min64(kTile, n - tl * kTile) * 4) & ~15u;
  };
  auto issue = [&](int64_t tl, int32_t *buf, uint64_t *b) {  // thread 0
    const uint32_t bytes = bulk_of(tl);
    if (!bytes) return;
    mbar_arrive_expect_tx(b, kScatter ? 2 * bytes : bytes);
    tma_load_1d(buf, loc + tl * kTile, bytes, b);
    if (kScatter) tma_load_1d(buf + kTile, in + tl * kTile, bytes, b);
  };
  for (int i = t; i < nwin; i += kThreads) scnt[i] = 0;
  if (t == 0) {
    s_total = 0;
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    for (int k = 0; k < 2; ++k)
      if (blockIdx.x + k * G < tiles) issue(blockIdx.x + k * G, bufs + k * 2 * kTile, &bar[k]);
  }
  __syncthreads();
  uint32_t phase = 0;
  int b = 0;
  int64_t tl = blockIdx.x;
  bool failed = false;
  for (; tl < tiles; tl += G, b ^= 1) {
    int32_t *buf = bufs + b * 2 * kTile;
    const int64_t base = tl * kTile;
    const int count = static_cast<int>(min64(kTile, n - base));
    const uint32_t bytes = bulk_of(tl);
    const int nb = static_cast<int>(bytes / 4);  // a multiple of 4
    bool bad = false;
    if (bytes) {
      bad = !mbar_wait_bounded(&bar[b], (phase >> b) & 1u, timeout_ns, fault);
      phase ^= 1u << b;
    }
    int2 pr[kPer];
    int wr[kPer];  // (window << 12) | rank, or -1 (kTile = 2^12 ranks)
#pragma unroll
    for (int k = 0; k < kPer / 4; ++k) {
      const int i0 = (k * kThreads + t) * 4;
      int32_t ls[4] = {-1, -1, -1, -1}, vs[4] = {0, 0, 0, 0};
      if (i0 < nb) {
        if (!bad) {
          const int4 l = *reinterpret_cast<const int4 *>(buf + i0);
          ls[0] = l.x, ls[1] = l.y, ls[2] = l.z, ls[3] = l.w;
          if (kScatter) {
            const int4 v = *reinterpret_cast<const int4 *>(buf + kTile + i0);
            vs[0] = v.x, vs[1] = v.y, vs[2] = v.z, vs[3] = v.w;
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (i0 + q < count) {
            ls[q] = loc[base + i0 + q];
            if (kScatter) vs[q] = in[base + i0 + q];
          }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int e = 4 * k + q;
        const bool valid = (i0 + q < count) && ls[q] >= 0 && static_cast<int64_t>(ls[q]) < n;
        const int w = ls[q] >> log_w;
        pr[e] = make_int2(ls[q], kScatter ? vs[q] : static_cast<int32_t>(base + i0 + q));
        wr[e] = valid ? (w << 12) | static_cast<int>(atomicAdd(&scnt[w], 1u)) : -1;
      }
    }
    if (__syncthreads_or(bad)) {  // A: counts complete; every read of buf done
      failed = true;
      break;
    }
    uint32_t g[MAXPER], o[MAXPER];
    claim_runs<MAXPER, kThreads>(scnt, soff, nwin, fill, &s_total, g, o);
    __syncthreads();  // B
    const uint32_t total = s_total;
    int2 *stage = reinterpret_cast<int2 *>(buf);
#pragma unroll
    for (int e = 0; e < kPer; ++e)
      if (wr[e] >= 0) stage[soff[wr[e] >> 12] + (wr[e] & (kTile - 1))] = pr[e];
    publish_run_bases<MAXPER, kThreads>(sgb, nwin, g, o);
    __syncthreads();  // C
    if (t == 0) s_total = 0;
    for (uint32_t s = t; s < total; s += kThreads) {
      const int2 p = stage[s];
      pairs[sgb[p.x >> log_w] + s] = p;
    }
    fence_proxy_async_smem();  // generic accesses of buf before the next bulk copy into it
    __syncthreads();
    if (t == 0 && tl + 2 * G < tiles) issue(tl + 2 * G, buf, &bar[b]);
  }
  if (failed && tl + G < tiles && bulk_of(tl + G))  // let the other buffer's copy land
    mbar_wait_bounded(&bar[b ^ 1], (phase >> (b ^ 1)) & 1u, timeout_ns, fault);
}

size_t part_pipe_smem(int nwin) {
  return 4 * static_cast<size_t>(kTile) * 4 + 3 * 4 * static_cast<size_t>(nwin);
}

// ---- gather fetch: ordered sweep, v = in[loc], regroup by destination --------------
__global__ void __launch_bounds__(kThreads)
    part_fetch_kernel(const int2 *__restrict__ pairs, const uint32_t *__restrict__ total_p,
                      const int32_t *__restrict__ in, int log_w, int nwin,
                      uint32_t *__restrict__ fill2, int2 *__restrict__ pairs2,
                      unsigned long long *ticket) {
  extern __shared__ __align__(16) unsigned char smem[];
  int2 *stage = reinterpret_cast<int2 *>(smem);
  uint32_t *scnt = reinterpret_cast<uint32_t *>(stage + kTile);
  uint32_t *soff = scnt + nwin;
  uint32_t *sgb = soff + nwin;
  __shared__ uint32_t s_warp[16];
  __shared__ int64_t s_chunk;
  const int64_t total = *total_p;
  const unsigned lt = lanemask_lt();
  const int t = threadIdx.x;
  while (true) {
    if (t == 0) s_chunk = static_cast<int64_t>(atomicAdd(ticket, 1ull));
    for (int i = t; i < nwin; i += kThreads) scnt[i] = 0;
    __syncthreads();
    const int64_t base = s_chunk * kTile;
    if (base >= total) break;
    int2 pr[kPer];
    int w[kPer], rank[kPer];
    // Pairs, 2 per 16-byte vector, row-striped; random loads all in flight.
    int2 src[kPer];
#pragma unroll
    for (int k = 0; k < kPer / 2; ++k) {
      const int64_t j = base + static_cast<int64_t>(k * kThreads + t) * 2;
      int4 q = make_int4(-1, 0, -1, 0);
      if (j + 1 < total) q = __ldcs(reinterpret_cast<const int4 *>(pairs + j));
      else if (j < total) { const int2 a = pairs[j]; q.x = a.x; q.y = a.y; }
      src[2 * k] = make_int2(q.x, q.y);
      src[2 * k + 1] = make_int2(q.z, q.w);
    }
#pragma unroll
    for (int e = 0; e < kPer; ++e) {
      const bool valid = src[e].x >= 0;
      pr[e] = make_int2(src[e].y, valid ? ld_random(in + src[e].x) : 0);  // {i, value}
    }
#pragma unroll
    for (int e = 0; e < kPer; ++e) {
      w[e] = src[e].x >= 0 ? (pr[e].x >> log_w) : -1;
      rank[e] = rank_in_window(w[e], scnt, lt);
    }
    __syncthreads();
    flush_runs<kPer>(pr, w, rank, nwin, log_w, scnt, soff, sgb, s_warp, stage, fill2, pairs2);
    __syncthreads();
  }
}

// ---- apply: ordered sweep, out[p.x] = p.y ------------------------------------------
// Scatter: pairs [0, total).  Gather: destination window j holds
// [j*W, fill2[j]).  chunks_per_win == 0 means the flat scatter layout.
__global__ void __launch_bounds__(kThreads)
    part_apply_kernel(const int2 *__restrict__ pairs, const uint32_t *__restrict__ total_p,
                      const uint32_t *__restrict__ fill2, int64_t w_elems, int64_t chunks_per_win,
                      int64_t num_chunks, int32_t *__restrict__ out, unsigned long long *ticket) {
  __shared__ int64_t s_chunk;
  const int t = threadIdx.x;
  while (true) {
    if (t == 0) s_chunk = static_cast<int64_t>(atomicAdd(ticket, 1ull));
    __syncthreads();
    const int64_t c = s_chunk;
    __syncthreads();
    if (c >= num_chunks) break;
    int64_t lo, hi;
    if (chunks_per_win == 0) {
      lo = c * kChunk;
      hi = min64(lo + kChunk, static_cast<int64_t>(*total_p));
    } else {
      const int64_t j = c / chunks_per_win, k = c % chunks_per_win;
      lo = j * w_elems + k * kChunk;
      hi = min64(lo + kChunk, static_cast<int64_t>(fill2[j]));
    }
    // 2 pairs per vector, 4 vectors per thread in flight.
    for (int64_t j0 = lo + 2 * t; j0 < hi; j0 += 2 * kThreads * 4) {
      int4 q[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t j = j0 + static_cast<int64_t>(u) * 2 * kThreads;
        q[u] = make_int4(-1, 0, -1, 0);
        if (j + 1 < hi) q[u] = __ldcs(reinterpret_cast<const int4 *>(pairs + j));
        else if (j < hi) { const int2 a = pairs[j]; q[u].x = a.x; q[u].y = a.y; }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (q[u].x >= 0) out[q[u].x] = q[u].y;
        if (q[u].z >= 0) out[q[u].z] = q[u].w;
      }
    }
  }
}

// ---- host side ---------------------------------------------------------------------
struct Plan {
  int log_w = 0;
  int nwin = 0;
  int64_t w_elems = 0;
};

int l2_bytes() {
  static std::once_flag once;
  static int bytes = 126 << 20;
  std::call_once(once, [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, dev) == cudaSuccess && v > 0)
      bytes = v;
  });
  return bytes;
}

// Windows of W = 2^k elements.  pass >= 2: W = next power of two >= ceil(n/pass);
// pass == 0: the largest W whose int32 slice fills at most half of L2.
Plan make_plan(int64_t n, int pass) {
  Plan p;
  int64_t w;
  if (pass <= 0) {
    w = 1;
    while (w * 2 * 4 <= l2_bytes() / 2) w *= 2;
  } else {
    const int64_t want = (n + pass - 1) / pass;
    w = 1;
    while (w < want) w *= 2;
  }
  if (w < kMinWin) w = kMinWin;  // keeps window starts 16-byte aligned in pairs2
  while ((n + w - 1) / w > kMaxWin) w *= 2;
  p.w_elems = w;
  p.log_w = 0;
  while ((int64_t(1) << p.log_w) < w) ++p.log_w;
  p.nwin = static_cast<int>((n + w - 1) / w);
  if (p.nwin < 1) p.nwin = 1;
  return p;
}

struct Layout {
  size_t cnt, fill, fill2, total, pairs, pairs2, bytes;
};

Layout layout_of(int64_t n, const Plan &p, bool gather) {
  Layout L{};
  size_t o = kHdr;
  auto take = [&](size_t b) {
    const size_t at = o;
    o += round_up(b, 256);
    return at;
  };
  L.cnt = take(4 * static_cast<size_t>(p.nwin));
  L.total = take(16);
  L.fill = take(4 * static_cast<size_t>(p.nwin));
  L.fill2 = gather ? take(4 * static_cast<size_t>(p.nwin)) : 0;
  L.pairs = take(8 * static_cast<size_t>(n));
  L.pairs2 = gather ? take(8 * static_cast<size_t>(p.nwin) * static_cast<size_t>(p.w_elems)) : 0;
  L.bytes = o;
  return L;
}

size_t part_smem(int nwin) { return static_cast<size_t>(kTile) * 8 + 3 * 4 * static_cast<size_t>(nwin); }

template <typename K> int set_smem(K kernel) {
  const size_t bytes = part_smem(kMaxWin);
  return cuda_status(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(bytes)));
}

int ensure_attrs() {
  static std::once_flag once[64];
  static int st[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::call_once(once[dev], [] {
    int d = 0;
    cudaGetDevice(&d);
    if (d < 0 || d >= 64) d = 0;
    int s = set_smem(part_partition_kernel<false>);
    if (s == EDPP_OK) s = set_smem(part_partition_kernel<true>);
    const int pipe_smem = static_cast<int>(part_pipe_smem(kMaxWin));
    auto pipe = [&](const void *k) {
      return cuda_status(
          cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, pipe_smem));
    };
    if (s == EDPP_OK) s = pipe(reinterpret_cast<const void *>(part_partition_pipe_kernel<false, 1>));
    if (s == EDPP_OK) s = pipe(reinterpret_cast<const void *>(part_partition_pipe_kernel<true, 1>));
    if (s == EDPP_OK)
      s = pipe(reinterpret_cast<const void *>(part_partition_pipe_kernel<false, kMaxWin / kThreads>));
    if (s == EDPP_OK)
      s = pipe(reinterpret_cast<const void *>(part_partition_pipe_kernel<true, kMaxWin / kThreads>));
    if (s == EDPP_OK) s = set_smem(part_fetch_kernel);
    st[d] = s;
  });
  return st[dev];
}

// The partition stage: pipelined when loc (and in) are 16-byte aligned.
template <bool kScatter>
int launch_partition(const int32_t *loc, const int32_t *in, int64_t n, int log_w, int nwin,
                     uint32_t *fill, int2 *pairs, bool vec, cudaStream_t st) {
  const int64_t tiles = (n + kTile - 1) / kTile;
  if (!vec) {
    part_partition_kernel<kScatter><<<static_cast<unsigned>(tiles), kThreads, part_smem(nwin), st>>>(
        loc, in, n, log_w, nwin, fill, pairs, false);
    return launch_status();
  }
  unsigned *fault = fault_word();
  if (!fault) return EDPP_ECUDA;
  const size_t smem = part_pipe_smem(nwin);
  auto run = [&](auto kernel) -> int {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem) != cudaSuccess)
      return EDPP_ECUDA;
    const int64_t blocks = min64(tiles, static_cast<int64_t>(device_sm_count()) * max64(per_sm, 1));
    kernel<<<static_cast<unsigned>(blocks), kThreads, smem, st>>>(loc, in, n, log_w, nwin, fill,
                                                                  pairs, kDefaultWaitNs, fault);
    return launch_status();
  };
  if (nwin <= kThreads) return run(part_partition_pipe_kernel<kScatter, 1>);
  return run(part_partition_pipe_kernel<kScatter, kMaxWin / kThreads>);
}

template <bool kScatter>
int part_run(const int32_t *in, int32_t *out, int64_t n, const int32_t *loc, int pass, void *ws,
             size_t ws_bytes, void *stream) {
  if (n < 0 || pass < 0) return EDPP_EINVAL;
  if (n == 0) return EDPP_OK;
  if (!in || !out || !loc) return EDPP_EINVAL;
  if (n > INT32_MAX) return EDPP_EINVAL;
  if (pass == 1) {  // one window: the direct single sweep is the partition
    return kScatter ? edpp_scatter_i32(in, out, n, loc, 1, stream)
                    : edpp_gather_i32(in, out, n, loc, 1, stream);
  }
  const Plan p = make_plan(n, pass);
  const Layout L = layout_of(n, p, !kScatter);
  if (!ws || ws_bytes < L.bytes) return EDPP_ENOMEM;
  int s = ensure_attrs();
  if (s != EDPP_OK) return s;
  cudaStream_t st = as_stream(stream);
  char *w = static_cast<char *>(ws);
  auto *tickets = reinterpret_cast<unsigned long long *>(w);
  auto *cnt = reinterpret_cast<uint32_t *>(w + L.cnt);
  auto *total = reinterpret_cast<uint32_t *>(w + L.total);
  auto *fill = reinterpret_cast<uint32_t *>(w + L.fill);
  auto *fill2 = kScatter ? nullptr : reinterpret_cast<uint32_t *>(w + L.fill2);
  auto *pairs = reinterpret_cast<int2 *>(w + L.pairs);
  auto *pairs2 = kScatter ? nullptr : reinterpret_cast<int2 *>(w + L.pairs2);
  if (cudaMemsetAsync(w, 0, L.fill, st) != cudaSuccess) return EDPP_ECUDA;  // tickets, cnt, total

  const int sms = device_sm_count();
  const bool vec_loc = aligned16(loc);
  const bool vec = vec_loc && (!kScatter || aligned16(in));
  const int64_t count_blocks = min64(static_cast<int64_t>(sms) * 8, (n + 4 * kThreads - 1) / (4 * kThreads));
  part_count_kernel<<<static_cast<unsigned>(max64(count_blocks, 1)), kThreads, 4 * p.nwin, st>>>(
      loc, n, p.log_w, p.nwin, cnt, vec_loc);
  part_bases_kernel<<<1, kThreads, 0, st>>>(cnt, fill, fill2, p.nwin, p.w_elems, total);
  const size_t smem = part_smem(p.nwin);
  s = launch_partition<kScatter>(loc, in, n, p.log_w, p.nwin, fill, pairs, vec, st);
  if (s != EDPP_OK) return s;
  const unsigned persist = static_cast<unsigned>(sms) * 4;
  if (kScatter) {
    const int64_t chunks = (n + kChunk - 1) / kChunk;  // upper bound; total <= n
    part_apply_kernel<<<persist, kThreads, 0, st>>>(pairs, total, nullptr, 0, 0, chunks, out,
                                                    tickets + 1);
  } else {
    part_fetch_kernel<<<persist, kThreads, smem, st>>>(pairs, total, in, p.log_w, p.nwin, fill2,
                                                       pairs2, tickets);
    const int64_t cpw = (p.w_elems + kChunk - 1) / kChunk;
    part_apply_kernel<<<persist, kThreads, 0, st>>>(pairs2, total, fill2, p.w_elems, cpw,
                                                    cpw * p.nwin, out, tickets + 1);
  }
  return launch_status();
}

// ==== shared-memory windows ("tiled" form) ===========================================
//
// The random side of the access moves from L2 into shared memory.  Pairs are
// partitioned twice by their key's window -- coarse windows of 128 fine
// windows, then fine windows of W = 2^14 (or 2^15) elements -- and one block
// per fine window applies its pairs inside a shared-memory copy of that
// window, so every global access is a streaming one:
//
//   scatter: count fine windows of loc -> scan -> partition {loc, in[i]} by
//            coarse window -> refine by fine window -> apply: per window,
//            out-window[loc - base] = value in shared memory, then store the
//            written elements of the window (bitmap), coalesced
//   gather:  count -> scan -> partition {loc, i} -> refine -> fetch: per
//            window of in[], load it once and emit {i, in[loc]} grouped by
//            the coarse window of i -> refine by fine window of i -> apply
//
// Streaming traffic per element: scatter ~48 B, gather ~80 B; no random
// global access.  Within a window, pairs arrive in no particular order (the
// per-window cursors are claimed atomically): every destination of a gather
// is written once; a scatter with repeated destinations keeps one of the
// colliding values, as the other forms do.
constexpr int kWinThreads = 512;
constexpr int kFineMinLog = 14;
constexpr int kFineMaxLog = 15;      // 32 K int32 = 128 KB window
constexpr int kMaxFine = 16384;      // count histogram: 64 KB of shared memory
constexpr int kCoarseLogFan = 7;     // 128 fine windows per coarse window

struct TPlan {
  int fine_log = kFineMinLog, coarse_log = kFineMinLog + kCoarseLogFan, F = 1, C = 1;
};

TPlan tplan(int64_t n) {
  TPlan p;
  while (((n + (int64_t{1} << p.fine_log) - 1) >> p.fine_log) > kMaxFine) ++p.fine_log;
  p.coarse_log = p.fine_log + kCoarseLogFan;
  p.F = static_cast<int>(max64(1, (n + (int64_t{1} << p.fine_log) - 1) >> p.fine_log));
  p.C = static_cast<int>(max64(1, (n + (int64_t{1} << p.coarse_log) - 1) >> p.coarse_log));
  return p;
}

bool tiled_fits(int64_t n) { return tplan(n).fine_log <= kFineMaxLog; }

__global__ void __launch_bounds__(kWinThreads)
    win_count_kernel(const int32_t *__restrict__ loc, int64_t n, int fine_log, int F,
                     uint32_t *__restrict__ cnt, bool vec) {
  extern __shared__ uint32_t hist[];
  for (int i = threadIdx.x; i < F; i += kWinThreads) hist[i] = 0;
  __syncthreads();
  const int64_t stride = static_cast<int64_t>(gridDim.x) * kWinThreads;
  const int64_t first = static_cast<int64_t>(blockIdx.x) * kWinThreads + threadIdx.x;
  auto add = [&](int32_t l) {
    if (static_cast<uint64_t>(static_cast<uint32_t>(l)) < static_cast<uint64_t>(n))
      atomicAdd(&hist[static_cast<uint32_t>(l) >> fine_log], 1u);
  };
  int64_t done = 0;
  if (vec) {
    const int64_t n4 = n >> 2;
    const int4 *l4 = reinterpret_cast<const int4 *>(loc);
    for (int64_t i = first; i < n4; i += stride) {
      const int4 q = __ldcs(l4 + i);
      add(q.x);
      add(q.y);
      add(q.z);
      add(q.w);
    }
    done = 4 * n4;
  }
  for (int64_t i = done + first; i < n; i += stride) add(loc[i]);
  __syncthreads();
  for (int i = threadIdx.x; i < F; i += kWinThreads)
    if (hist[i]) atomicAdd(&cnt[i], hist[i]);
}

// start[f] = sum of cnt[0..f), start[F] = total; fill = start; cfill[c] =
// start[c * 128]; gather also gets fill2[f] = f * W and cfill2[c] = c * 128 W.
__global__ void __launch_bounds__(1024)
    win_scan_kernel(const uint32_t *__restrict__ cnt, int F, int C, int fine_log, int coarse_log,
                    uint32_t *__restrict__ start, uint32_t *__restrict__ fill,
                    uint32_t *__restrict__ cfill, uint32_t *__restrict__ fill2,
                    uint32_t *__restrict__ cfill2) {
  __shared__ uint32_t wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (F + 1023) / 1024;  // <= kMaxFine / 1024
  const int lo = min(F, t * per), hi = min(F, lo + per);
  // all of this thread's counts are loaded at once and kept in registers
  constexpr int kPerMax = kMaxFine / 1024;
  uint32_t v[kPerMax];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kPerMax; ++k) {
    v[k] = lo + k < hi ? cnt[lo + k] : 0u;
    s += v[k];
  }
  uint32_t incl = s;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    const uint32_t x = wsum[lane];
    uint32_t xi = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, xi, d);
      if (lane >= d) xi += y;
    }
    wsum[lane] = xi - x;
    if (lane == 31) start[F] = xi;
  }
  __syncthreads();
  uint32_t run = wsum[w] + incl - s;
#pragma unroll
  for (int k = 0; k < kPerMax; ++k) {
    const int i = lo + k;
    if (i < hi) {
      start[i] = run;
      fill[i] = run;
      if ((i & ((1 << kCoarseLogFan) - 1)) == 0) cfill[i >> kCoarseLogFan] = run;
      run += v[k];
    }
  }
  if (fill2) {
    for (int i = t; i < F; i += 1024) fill2[i] = static_cast<uint32_t>(i) << fine_log;
    for (int c = t; c < C; c += 1024) cfill2[c] = static_cast<uint32_t>(c) << coarse_log;
  }
}

// Append every pair of one tile to fine window (pair.x >> fine_log) at that
// window's cursor, as two arrays: the offset of pair.x inside its window
// (16 bits: windows are at most 2^15 elements) and pair.y.  Six bytes per
// pair instead of eight, on the write here and on the read of every later
// stage.  The tiles ("slots") are either the flat range [0, *total)
// cut into kTile pairs, or, with region_log > 0, each region
// [r << region_log, region_end[r]) cut the same way (slots past a region's
// end are empty).  Either way the pairs are ordered by coarse window
// (pair.x >> coarse_log), so a slot's fine windows lie in the coarse windows
// of its first and last pair.  Persistent blocks take slots blockIdx,
// +gridDim, ...; the slot after next is copied into shared memory by TMA
// while the current one is processed, so loads stay in flight through the
// block's grouping work.  A slot whose fine windows span at most kRefineSpan
// is grouped in shared memory (the landed input buffer is reused as the
// staging area) and written as one run per window; a wider one (skewed keys)
// appends pair by pair.
constexpr int kRefineSpan = 512;
constexpr int kRefineBlocksPerSm = 3;

__device__ __forceinline__ void refine_range(int64_t slot, const uint32_t *total_p,
                                             const uint32_t *region_end, int region_log,
                                             int64_t &lo, int64_t &hi) {
  if (region_log > 0) {
    const int shift = region_log - 12;  // kTile = 4096 = 2^12
    const int64_t r = slot >> shift;
    lo = (r << region_log) + ((slot & ((int64_t{1} << shift) - 1)) << 12);
    hi = min64(lo + kTile, static_cast<int64_t>(region_end[r]));
  } else {
    lo = slot * kTile;
    hi = min64(lo + kTile, static_cast<int64_t>(*total_p));
  }
}

// Thread 0: start the bulk copy of the even part of [lo, hi) into buf.
__device__ __forceinline__ void refine_issue(const int2 *src, int64_t lo, int64_t hi, int2 *buf,
                                             uint64_t *bar) {
  const uint32_t even = static_cast<uint32_t>(hi - lo) & ~1u;
  if (lo < hi && even) {
    mbar_arrive_expect_tx(bar, even * 8u);
    tma_load_1d(buf, src + lo, even * 8u, bar);
  }
}

__global__ void __launch_bounds__(kThreads, kRefineBlocksPerSm)
    win_refine_kernel(const int2 *__restrict__ src, const uint32_t *__restrict__ total_p,
                      const uint32_t *__restrict__ region_end, int region_log, int fine_log,
                      int coarse_log, int64_t slots, uint32_t *__restrict__ fill,
                      uint16_t *__restrict__ dst_off, int32_t *__restrict__ dst_val,
                      uint64_t timeout_ns, unsigned *fault) {
  extern __shared__ __align__(16) unsigned char smem[];
  int2 *bufs = reinterpret_cast<int2 *>(smem);  // [2][kTile]
  uint32_t *scnt = reinterpret_cast<uint32_t *>(bufs + 2 * kTile);
  uint32_t *soff = scnt + kRefineSpan;
  uint32_t *sgb = soff + kRefineSpan;
  __shared__ alignas(8) uint64_t bar[2];
  __shared__ uint32_t s_total;
  const int t = threadIdx.x;
  const int64_t G = gridDim.x;
  const int fan = coarse_log - fine_log;
  const uint32_t wmask = (1u << fine_log) - 1u;
  for (int i = t; i < kRefineSpan; i += kThreads) scnt[i] = 0;
  if (t == 0) {
    s_total = 0;
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    for (int k = 0; k < 2; ++k) {
      const int64_t sk = blockIdx.x + k * G;
      if (sk < slots) {
        int64_t lo, hi;
        refine_range(sk, total_p, region_end, region_log, lo, hi);
        refine_issue(src, lo, hi, bufs + k * kTile, &bar[k]);
      }
    }
  }
  __syncthreads();
  uint32_t phase = 0;  // bit b: parity of bar[b]'s next completion
  int b = 0;
  int64_t slot = blockIdx.x;
  bool failed = false;
  for (; slot < slots; slot += G, b ^= 1) {
    int64_t lo, hi;
    refine_range(slot, total_p, region_end, region_log, lo, hi);
    int2 *buf = bufs + b * kTile;
    if (lo < hi) {  // block-uniform
      const uint32_t cnt = static_cast<uint32_t>(hi - lo);
      const uint32_t even = cnt & ~1u;  // pairs in the bulk copy; an odd last one is read from src
      bool bad = false;
      if (even) {
        bad = !mbar_wait_bounded(&bar[b], (phase >> b) & 1u, timeout_ns, fault);
        phase ^= 1u << b;
      }
      int wlo = 0, span = 0;
      if (!bad) {
        const int2 first = even ? buf[0] : src[lo];
        const int2 last = (cnt & 1u) ? src[hi - 1] : buf[cnt - 1];
        const int c0 = first.x >> coarse_log, c1 = last.x >> coarse_log;
        wlo = c0 << fan;
        span = (c1 - c0 + 1) << fan;
      }
      const bool grouped = span <= kRefineSpan;  // uniform unless bad
      int2 pr[kPer];
      int fid[kPer];
#pragma unroll
      for (int k = 0; k < kPer / 2; ++k) {
        const uint32_t j = static_cast<uint32_t>(k * kThreads + t) * 2u;
        int4 q = make_int4(0, 0, 0, 0);
        if (j < even) {
          if (!bad) q = *reinterpret_cast<const int4 *>(buf + j);
        } else if (j < cnt) {
          const int2 a = src[lo + j];
          q.x = a.x;
          q.y = a.y;
        }
        pr[2 * k] = make_int2(q.x, q.y);
        pr[2 * k + 1] = make_int2(q.z, q.w);
        fid[2 * k] = (j < cnt && !bad) ? (q.x >> fine_log) - wlo : -1;
        fid[2 * k + 1] = (j + 1 < cnt && !bad) ? (q.z >> fine_log) - wlo : -1;
      }
      // fid[e] becomes (window << 12) | rank, or -1 (kTile = 2^12 ranks)
      if (grouped) {
#pragma unroll
        for (int e = 0; e < kPer; ++e)
          if (fid[e] >= 0) fid[e] = (fid[e] << 12) | static_cast<int>(atomicAdd(&scnt[fid[e]], 1u));
      }
      if (__syncthreads_or(bad)) {  // A: ranks complete; every read of buf done
        failed = true;
        break;
      }
      if (!grouped) {  // skewed slot: one cursor claim per pair
#pragma unroll
        for (int e = 0; e < kPer; ++e)
          if (fid[e] >= 0) {
            const uint32_t idx = atomicAdd(&fill[wlo + fid[e]], 1u);
            dst_off[idx] = static_cast<uint16_t>(static_cast<uint32_t>(pr[e].x) & wmask);
            dst_val[idx] = pr[e].y;
          }
      } else {
        uint32_t g[kRefineSpan / kThreads], o[kRefineSpan / kThreads];
        claim_runs<kRefineSpan / kThreads, kThreads>(scnt, soff, span, fill + wlo, &s_total, g, o);
        __syncthreads();  // B
        const uint32_t total = s_total;
#pragma unroll
        for (int e = 0; e < kPer; ++e)
          if (fid[e] >= 0) buf[soff[fid[e] >> 12] + (fid[e] & (kTile - 1))] = pr[e];
        publish_run_bases<kRefineSpan / kThreads, kThreads>(sgb, span, g, o);
        __syncthreads();  // C
        if (t == 0) s_total = 0;
        for (uint32_t q = t; q < total; q += kThreads) {
          const int2 p = buf[q];
          const uint32_t idx = sgb[(p.x >> fine_log) - wlo] + q;
          dst_off[idx] = static_cast<uint16_t>(static_cast<uint32_t>(p.x) & wmask);
          dst_val[idx] = p.y;
        }
      }
      fence_proxy_async_smem();  // generic accesses of buf before the next bulk copy into it
      __syncthreads();
    }
    if (t == 0) {
      const int64_t sn = slot + 2 * G;
      if (sn < slots) {
        int64_t lo2, hi2;
        refine_range(sn, total_p, region_end, region_log, lo2, hi2);
        refine_issue(src, lo2, hi2, buf, &bar[b]);
      }
    }
  }
  if (failed) {
    // let the other buffer's copy (slot + G), if one was started, land
    const int64_t sn = slot + G;
    if (sn < slots) {
      int64_t lo2, hi2;
      refine_range(sn, total_p, region_end, region_log, lo2, hi2);
      if (lo2 < hi2 && ((static_cast<uint32_t>(hi2 - lo2) & ~1u) != 0u))
        mbar_wait_bounded(&bar[b ^ 1], (phase >> (b ^ 1)) & 1u, timeout_ns, fault);
    }
  }
}

// One block per fine window f: pairs [start[f], start[f+1]) (or, without
// start, [f << fine_log, fill_end[f])) are {offset in the window, value}
// (two arrays, as the refine writes them); they are applied in shared memory and the written elements of
// the window are stored (a bitmap marks them; untouched elements keep their
// old value in `out`).  unique: no index repeats (a gather's return trip),
// so a window with as many pairs as elements is written whole and needs no
// bitmap.
__global__ void __launch_bounds__(kWinThreads)
    win_apply_kernel(const uint16_t *__restrict__ poff, const int32_t *__restrict__ pval,
                     const uint32_t *__restrict__ start, const uint32_t *__restrict__ fill_end,
                     int fine_log, int64_t n, int32_t *__restrict__ out, bool vec_out,
                     bool unique) {
  extern __shared__ __align__(16) int32_t win[];
  const int W = 1 << fine_log;
  uint32_t *bits = reinterpret_cast<uint32_t *>(win + W);
  const int f = blockIdx.x;
  const int64_t base = static_cast<int64_t>(f) << fine_log;
  const int len = static_cast<int>(min64(W, n - base));
  const int64_t lo = start ? start[f] : base;
  const int64_t hi = start ? start[f + 1] : fill_end[f];
  const bool whole = unique && hi - lo == len;  // block-uniform
  const int t = threadIdx.x;
  if (!whole)
    for (int i = t; i < (W >> 5); i += kWinThreads) bits[i] = 0u;
  __syncthreads();
  auto put = [&](uint32_t rel, int32_t v) {
    win[rel] = v;
    if (!whole) atomicOr(&bits[rel >> 5], 1u << (rel & 31));
  };
  // pairs: a scalar head up to a multiple of 8, then groups of 8 (one 16-byte
  // load of offsets, two of values; both arrays are 16-byte aligned), then a
  // scalar tail
  const int64_t head = min64(hi, (lo + 7) & ~int64_t{7});
  for (int64_t q = lo + t; q < head; q += kWinThreads) put(poff[q], pval[q]);
  const int64_t ng = (hi - head) >> 3;
  const uint4 *o4 = reinterpret_cast<const uint4 *>(poff + head);
  const uint4 *v4 = reinterpret_cast<const uint4 *>(pval + head);
  for (int64_t g = t; g < ng; g += 2 * kWinThreads) {
    uint4 qo[2], qv[4];
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (g + u * kWinThreads < ng) {
        qo[u] = __ldcs(o4 + g + u * kWinThreads);
        qv[2 * u] = __ldcs(v4 + 2 * (g + u * kWinThreads));
        qv[2 * u + 1] = __ldcs(v4 + 2 * (g + u * kWinThreads) + 1);
      }
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (g + u * kWinThreads < ng) {
        const uint32_t os[4] = {qo[u].x, qo[u].y, qo[u].z, qo[u].w};
        const uint32_t vs[8] = {qv[2 * u].x, qv[2 * u].y, qv[2 * u].z, qv[2 * u].w,
                                qv[2 * u + 1].x, qv[2 * u + 1].y, qv[2 * u + 1].z,
                                qv[2 * u + 1].w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          put(os[k] & 0xffffu, static_cast<int32_t>(vs[2 * k]));
          put(os[k] >> 16, static_cast<int32_t>(vs[2 * k + 1]));
        }
      }
  }
  for (int64_t q = head + 8 * ng + t; q < hi; q += kWinThreads) put(poff[q], pval[q]);
  __syncthreads();
  for (int e0 = 4 * t; e0 < len; e0 += 4 * kWinThreads) {
    const uint32_t nib = whole ? 0xFu : (bits[e0 >> 5] >> (e0 & 31)) & 0xFu;
    if (nib == 0xFu && vec_out && e0 + 3 < len) {
      __stcs(reinterpret_cast<int4 *>(out + base + e0), *reinterpret_cast<const int4 *>(win + e0));
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (e0 + k < len && ((nib >> k) & 1u)) out[base + e0 + k] = win[e0 + k];
    }
  }
}

// Gather fetch: one block per fine window f of in[]; the window is loaded
// once into shared memory, and each pair {loc, i} of the window (the offset
// of loc in the window and i, in two arrays) becomes
// {i, in[loc]}, appended to the coarse window of i (cursors cfill2).  The
// window's pairs go in sub-tiles of kTile; each sub-tile's pairs are loaded
// into registers while the previous one is grouped (the first while the
// window lands).
constexpr int kFetchThreads = 512;
constexpr int kFetchPer = kTile / kFetchThreads;  // 8 pairs per thread per sub-tile

__global__ void __launch_bounds__(kFetchThreads)
    win_fetch_kernel(const uint16_t *__restrict__ poff, const int32_t *__restrict__ pidx,
                     const uint32_t *__restrict__ start,
                     const int32_t *__restrict__ in, int64_t n, int fine_log, int coarse_log,
                     int C, uint32_t *__restrict__ cfill2, int2 *__restrict__ dst, bool vec_in,
                     uint64_t timeout_ns, unsigned *fault) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int W = 1 << fine_log;
  int32_t *win = reinterpret_cast<int32_t *>(smem);
  int2 *stage = reinterpret_cast<int2 *>(win + W);
  uint32_t *scnt = reinterpret_cast<uint32_t *>(stage + kTile);
  uint32_t *soff = scnt + C;
  uint32_t *sgb = soff + C;
  __shared__ uint32_t s_total;
  __shared__ alignas(8) uint64_t bar;
  const int f = blockIdx.x, t = threadIdx.x;
  const int64_t base = static_cast<int64_t>(f) << fine_log;
  const int len = static_cast<int>(min64(W, n - base));
  const int64_t lo = start[f], hi = start[f + 1];
  if (lo >= hi) return;  // block-uniform
  uint32_t nxt_off[kFetchPer];
  int32_t nxt_i[kFetchPer];
  auto load = [&](int64_t c0) {
#pragma unroll
    for (int e = 0; e < kFetchPer; ++e) {
      const int64_t j = c0 + static_cast<int64_t>(e) * kFetchThreads + t;
      nxt_off[e] = j < hi ? __ldcs(poff + j) : 0u;
      nxt_i[e] = j < hi ? __ldcs(pidx + j) : 0;
    }
  };
  // the window by one bulk copy (16-byte multiple), the rest by plain loads
  const uint32_t bulk = vec_in ? (static_cast<uint32_t>(len) * 4u) & ~15u : 0u;
  if (t == 0 && bulk) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_arrive_expect_tx(&bar, bulk);
    tma_load_1d(win, in + base, bulk, &bar);
  }
  load(lo);
  for (int e = static_cast<int>(bulk / 4) + t; e < len; e += kFetchThreads) win[e] = in[base + e];
  for (int i = t; i < C; i += kFetchThreads) scnt[i] = 0;
  if (t == 0) s_total = 0;
  __syncthreads();  // barrier initialised before anyone waits on it
  if (bulk && __syncthreads_or(!mbar_wait_bounded(&bar, 0, timeout_ns, fault))) return;
  for (int64_t c0 = lo; c0 < hi; c0 += kTile) {
    uint32_t ao[kFetchPer];
    int32_t ai[kFetchPer];
#pragma unroll
    for (int e = 0; e < kFetchPer; ++e) {
      ao[e] = nxt_off[e];
      ai[e] = nxt_i[e];
    }
    if (c0 + kTile < hi) load(c0 + kTile);
    int2 pr[kFetchPer];
    int w[kFetchPer], rank[kFetchPer];
#pragma unroll
    for (int e = 0; e < kFetchPer; ++e) {
      const bool valid = c0 + static_cast<int64_t>(e) * kFetchThreads + t < hi;
      pr[e] = make_int2(ai[e], valid ? win[ao[e]] : 0);  // {i, value}
      w[e] = valid ? (ai[e] >> coarse_log) : -1;
      rank[e] = valid ? static_cast<int>(atomicAdd(&scnt[w[e]], 1u)) : -1;
    }
    __syncthreads();  // A
    uint32_t g[1], o[1];
    claim_runs<1, kFetchThreads>(scnt, soff, C, cfill2, &s_total, g, o);
    __syncthreads();  // B
    const uint32_t total = s_total;
#pragma unroll
    for (int e = 0; e < kFetchPer; ++e)
      if (w[e] >= 0) stage[soff[w[e]] + rank[e]] = pr[e];
    publish_run_bases<1, kFetchThreads>(sgb, C, g, o);
    __syncthreads();  // C
    if (t == 0) s_total = 0;
    for (uint32_t q = t; q < total; q += kFetchThreads) {
      const int2 p = stage[q];
      dst[sgb[p.x >> coarse_log] + q] = p;
    }
  }
}

size_t refine_smem() {
  return 2 * static_cast<size_t>(kTile) * 8 + 3 * 4 * static_cast<size_t>(kRefineSpan);
}
size_t apply_smem(int fine_log) { return (size_t{4} << fine_log) + (size_t{1} << fine_log) / 8; }
size_t fetch_smem(int fine_log, int C) {
  return (size_t{4} << fine_log) + static_cast<size_t>(kTile) * 8 + 3 * 4 * static_cast<size_t>(C);
}

int ensure_win_attrs() {
  static std::once_flag once[64];
  static int st[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::call_once(once[dev], [dev] {
    auto set = [](const void *k, size_t b) {
      return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(b));
    };
    cudaError_t e = set(reinterpret_cast<const void *>(win_count_kernel), 4 * kMaxFine);
    if (e == cudaSuccess) e = set(reinterpret_cast<const void *>(win_refine_kernel), refine_smem());
    if (e == cudaSuccess) e = set(reinterpret_cast<const void *>(win_apply_kernel), apply_smem(kFineMaxLog));
    if (e == cudaSuccess)
      e = set(reinterpret_cast<const void *>(win_fetch_kernel), fetch_smem(kFineMaxLog, 1 << (31 - kFineMaxLog - kCoarseLogFan)));
    if (e == cudaSuccess)
      e = set(reinterpret_cast<const void *>(part_partition_kernel<true>), part_smem(kMaxWin));
    if (e == cudaSuccess)
      e = set(reinterpret_cast<const void *>(part_partition_kernel<false>), part_smem(kMaxWin));
    st[dev] = e == cudaSuccess ? EDPP_OK : EDPP_ECUDA;
  });
  return st[dev];
}

// pairs_a: 8-byte pairs {x, y} (partition and fetch output); pairs_b: the
// refine's output as 16-bit window offsets (at pairs_b) and 32-bit values
// (at pairs_b + soa_val), both 16-byte aligned.
struct TLayout {
  size_t cnt, start, fill, cfill, fill2, cfill2, pairs_a, pairs_b, soa_val, bytes;
};

TLayout tlayout_of(int64_t n, const TPlan &p, bool gather) {
  TLayout L{};
  size_t o = kHdr;
  auto take = [&](size_t b) {
    const size_t at = o;
    o += round_up(b, 256);
    return at;
  };
  L.cnt = take(4 * static_cast<size_t>(p.F));
  L.start = take(4 * static_cast<size_t>(p.F + 1));
  L.fill = take(4 * static_cast<size_t>(p.F));
  L.cfill = take(4 * static_cast<size_t>(p.C));
  L.fill2 = gather ? take(4 * static_cast<size_t>(p.F)) : 0;
  L.cfill2 = gather ? take(4 * static_cast<size_t>(p.C)) : 0;
  L.pairs_a = take(8 * static_cast<size_t>(n));
  L.soa_val = round_up(2 * static_cast<size_t>(n), 256);
  L.pairs_b = take(L.soa_val + 4 * static_cast<size_t>(n));
  L.bytes = o;
  return L;
}

template <bool kScatter>
int tiled_run(const int32_t *in, int32_t *out, int64_t n, const int32_t *loc, int pass, void *ws,
              size_t ws_bytes, void *stream) {
  if (n < 0 || pass < 0) return EDPP_EINVAL;
  if (n == 0) return EDPP_OK;
  if (!in || !out || !loc) return EDPP_EINVAL;
  if (n > INT32_MAX) return EDPP_EINVAL;
  if (!tiled_fits(n)) return part_run<kScatter>(in, out, n, loc, 0, ws, ws_bytes, stream);
  const TPlan p = tplan(n);
  const TLayout L = tlayout_of(n, p, !kScatter);
  if (!ws || ws_bytes < L.bytes) return EDPP_ENOMEM;
  int s = ensure_win_attrs();
  if (s == EDPP_OK) s = ensure_attrs();
  if (s != EDPP_OK) return s;
  cudaStream_t st = as_stream(stream);
  char *w = static_cast<char *>(ws);
  auto *cnt = reinterpret_cast<uint32_t *>(w + L.cnt);
  auto *start = reinterpret_cast<uint32_t *>(w + L.start);
  auto *fill = reinterpret_cast<uint32_t *>(w + L.fill);
  auto *cfill = reinterpret_cast<uint32_t *>(w + L.cfill);
  auto *fill2 = kScatter ? nullptr : reinterpret_cast<uint32_t *>(w + L.fill2);
  auto *cfill2 = kScatter ? nullptr : reinterpret_cast<uint32_t *>(w + L.cfill2);
  auto *pa = reinterpret_cast<int2 *>(w + L.pairs_a);
  auto *pb_off = reinterpret_cast<uint16_t *>(w + L.pairs_b);
  auto *pb_val = reinterpret_cast<int32_t *>(w + L.pairs_b + L.soa_val);
  if (cudaMemsetAsync(cnt, 0, 4 * static_cast<size_t>(p.F), st) != cudaSuccess) return EDPP_ECUDA;
  const int sms = device_sm_count();
  const bool vec_loc = aligned16(loc);
  const bool vec_in = aligned16(in);
  const int64_t cblocks = min64(static_cast<int64_t>(sms) * 2, (n + 4 * kWinThreads - 1) / (4 * kWinThreads));
  win_count_kernel<<<static_cast<unsigned>(max64(cblocks, 1)), kWinThreads, 4 * p.F, st>>>(
      loc, n, p.fine_log, p.F, cnt, vec_loc);
  win_scan_kernel<<<1, 1024, 0, st>>>(cnt, p.F, p.C, p.fine_log, p.coarse_log, start, fill, cfill,
                                      fill2, cfill2);
  const int64_t tiles = (n + kTile - 1) / kTile;
  s = launch_partition<kScatter>(loc, in, n, p.coarse_log, p.C, cfill, pa,
                                 vec_loc && (!kScatter || vec_in), st);
  if (s != EDPP_OK) return s;
  unsigned *fault = fault_word();
  if (!fault) return EDPP_ECUDA;
  const int64_t rblocks = static_cast<int64_t>(sms) * kRefineBlocksPerSm;
  win_refine_kernel<<<static_cast<unsigned>(min64(tiles, rblocks)), kThreads, refine_smem(), st>>>(
      pa, start + p.F, nullptr, 0, p.fine_log, p.coarse_log, tiles, fill, pb_off, pb_val,
      kDefaultWaitNs, fault);
  if (kScatter) {
    win_apply_kernel<<<static_cast<unsigned>(p.F), kWinThreads, apply_smem(p.fine_log), st>>>(
        pb_off, pb_val, start, nullptr, p.fine_log, n, out, aligned16(out), false);
  } else {
    win_fetch_kernel<<<static_cast<unsigned>(p.F), kFetchThreads, fetch_smem(p.fine_log, p.C), st>>>(
        pb_off, pb_val, start, in, n, p.fine_log, p.coarse_log, p.C, cfill2, pa, vec_in,
        kDefaultWaitNs, fault);
    const int64_t rtiles = static_cast<int64_t>(p.C) << (p.coarse_log - 12);
    win_refine_kernel<<<static_cast<unsigned>(min64(rtiles, rblocks)), kThreads, refine_smem(), st>>>(
        pa, nullptr, cfill2, p.coarse_log, p.fine_log, p.coarse_log, rtiles, fill2, pb_off, pb_val,
        kDefaultWaitNs, fault);
    win_apply_kernel<<<static_cast<unsigned>(p.F), kWinThreads, apply_smem(p.fine_log), st>>>(
        pb_off, pb_val, nullptr, fill2, p.fine_log, n, out, aligned16(out), true);
  }
  return launch_status();
}

}  // namespace
}  // namespace edpp

extern "C" {

size_t edpp_gather_workspace_size(int64_t length, int pass) {
  if (length <= 0 || pass < 0 || pass == 1) return 0;
  return edpp::layout_of(length, edpp::make_plan(length, pass), true).bytes;
}

size_t edpp_scatter_workspace_size(int64_t length, int pass) {
  if (length <= 0 || pass < 0 || pass == 1) return 0;
  return edpp::layout_of(length, edpp::make_plan(length, pass), false).bytes;
}

int edpp_gather_i32_ws(const int32_t *in, int32_t *out, int64_t length, const int32_t *loc,
                       int pass, void *ws, size_t ws_bytes, void *stream) {
  return edpp::part_run<false>(in, out, length, loc, pass, ws, ws_bytes, stream);
}

int edpp_scatter_i32_ws(const int32_t *in, int32_t *out, int64_t length, const int32_t *loc,
                        int pass, void *ws, size_t ws_bytes, void *stream) {
  return edpp::part_run<true>(in, out, length, loc, pass, ws, ws_bytes, stream);
}

size_t edpp_gather_tiled_workspace_size(int64_t length) {
  if (length <= 0) return 0;
  if (!edpp::tiled_fits(length)) return edpp_gather_workspace_size(length, 0);
  return edpp::tlayout_of(length, edpp::tplan(length), true).bytes;
}

size_t edpp_scatter_tiled_workspace_size(int64_t length) {
  if (length <= 0) return 0;
  if (!edpp::tiled_fits(length)) return edpp_scatter_workspace_size(length, 0);
  return edpp::tlayout_of(length, edpp::tplan(length), false).bytes;
}

int edpp_gather_i32_tiled(const int32_t *in, int32_t *out, int64_t length, const int32_t *loc,
                          int pass, void *ws, size_t ws_bytes, void *stream) {
  return edpp::tiled_run<false>(in, out, length, loc, pass, ws, ws_bytes, stream);
}

int edpp_scatter_i32_tiled(const int32_t *in, int32_t *out, int64_t length, const int32_t *loc,
                           int pass, void *ws, size_t ws_bytes, void *stream) {
  return edpp::tiled_run<true>(in, out, length, loc, pass, ws, ws_bytes, stream);
}

int edpp_gather_prefers_direct(int64_t length) {
  // Without a tuning entry: a gather whose source is at most ~2.5x L2 keeps
  // enough of it in L2 that the direct random sweep wins (measured, int32
  // permutations: 2^25 0.49 ms direct against 0.59 ms tiled; 2^26 1.00
  // against 1.10; 2^28 5.34 against 4.32).
  const bool rule =
      static_cast<double>(length) * 4.0 <= 2.5 * static_cast<double>(edpp::device_l2_bytes());
  return edpp::tuned_variant(EDPP_TUNE_GATHER, 4, length, rule ? 1 : 0) == 1;
}

}  // extern "C"
