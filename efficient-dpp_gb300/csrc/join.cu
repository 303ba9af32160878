// join.cu — partitioned hash join (match count) on the stable split.
//
// Follows the reference's partitioned hash join
// (obsolete/OpenCL/phjImpl.cpp:14-129, hj_partitioned_kernel.cl:8-107):
// both relations are split into B buckets by key & (B-1), then one block per
// bucket builds an open-addressing table from the S partition in shared
// memory and probes it with the R partition, counting pairs with equal keys
// (the reference only counts, res_len).  GB300 form: the partitions come from
// edpp_split_i32 (keys only, bucket starts from its histogram); the table
// holds 64-bit slots {count, key} set by shared-memory atomicCAS; an S
// partition larger than half the table is processed in chunks (build chunk,
// probe all of R's partition, repeat), so any skew stays exact.  The count is
// sum over keys of count_R(key) * count_S(key).
#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace edpp {
namespace {

constexpr int kThreads = 1024;  // one block per SM (128 KB table): 32 warps hide its latency
                                // (512 threads: 3.31 against 2.51 ms for 2^26 x 2^26)
constexpr int kTableLog2 = 14;              // 16384 slots x 8 bytes = 128 KB
constexpr int kTable = 1 << kTableLog2;
constexpr int kChunk = kTable / 2;          // S tuples per build (load <= 0.5)

__device__ __forceinline__ uint32_t slot_of(int32_t key) {
  // multiplicative hash on the bits above the partition bits' influence
  return (static_cast<uint32_t>(key) * 0x9E3779B1u) >> (32 - kTableLog2);
}

__global__ void __launch_bounds__(kThreads)
    join_probe_kernel(const int32_t *__restrict__ r_keys, int64_t r_len,
                      const int32_t *__restrict__ r_start, const int32_t *__restrict__ s_keys,
                      int64_t s_len, const int32_t *__restrict__ s_start, int buckets,
                      unsigned long long *__restrict__ count) {
  extern __shared__ unsigned long long table[];  // kTable slots
  __shared__ unsigned long long s_red[kThreads / 32];
  const int b = blockIdx.x;
  const int64_t r_lo = r_start[b], r_hi = b + 1 < buckets ? r_start[b + 1] : r_len;
  const int64_t s_lo = s_start[b], s_hi = b + 1 < buckets ? s_start[b + 1] : s_len;
  unsigned long long matches = 0;
  for (int64_t c0 = s_lo; c0 < s_hi; c0 += kChunk) {
    const int64_t c1 = min64(s_hi, c0 + kChunk);
    for (int i = threadIdx.x; i < kTable; i += kThreads) table[i] = 0ull;
    __syncthreads();
    // build: a slot is {count:32 | key:32}; equal keys share one slot and
    // bump its count, so duplicate-heavy partitions keep short probe chains.
    // A claimed slot's key never changes, so the CAS result identifies it.
    for (int64_t i = c0 + threadIdx.x; i < c1; i += kThreads) {
      const uint32_t key = static_cast<uint32_t>(s_keys[i]);
      const unsigned long long entry = (1ull << 32) | key;
      uint32_t h = slot_of(static_cast<int32_t>(key));
      while (true) {
        const unsigned long long cur = atomicCAS(&table[h], 0ull, entry);
        if (cur == 0ull) break;
        if (static_cast<uint32_t>(cur) == key) {
          atomicAdd(&table[h], 1ull << 32);
          break;
        }
        h = (h + 1) & (kTable - 1);
      }
    }
    __syncthreads();
    // probe: at most one slot holds the key; stop at it or at an empty slot
    for (int64_t i = r_lo + threadIdx.x; i < r_hi; i += kThreads) {
      const uint32_t key = static_cast<uint32_t>(r_keys[i]);
      uint32_t h = slot_of(static_cast<int32_t>(key));
      unsigned long long e;
      while ((e = table[h]) != 0ull) {
        if (static_cast<uint32_t>(e) == key) {
          matches += e >> 32;
          break;
        }
        h = (h + 1) & (kTable - 1);
      }
    }
    __syncthreads();
  }
  // block sum
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) matches += __shfl_xor_sync(0xffffffffu, matches, m);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = matches;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < kThreads / 32; ++w) t += s_red[w];
    if (t) atomicAdd(count, t);
  }
}

// ---- non-partitioned form: one table in HBM/L2 -------------------------------
// (obsolete/OpenCL/nphjImpl.cpp:15-144, hj_non_partitioned_kernel.cl:9-77):
// build a table of 2^bits >= 2*|build side| slots, then every probe tuple walks
// its chain.  Same {count, key} slots as the shared-memory table; a 129 MB L2
// holds the table for build sides up to about 4M tuples.
__device__ __forceinline__ uint32_t np_slot(uint32_t key, int bits) {
  return (key * 0x9E3779B1u) >> (32 - bits);
}

__global__ void __launch_bounds__(256)
    join_np_build_kernel(const int32_t *__restrict__ keys, int64_t n,
                         unsigned long long *__restrict__ table, int bits) {
  const uint32_t mask = (1u << bits) - 1u;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t key = static_cast<uint32_t>(keys[i]);
    const unsigned long long entry = (1ull << 32) | key;
    uint32_t h = np_slot(key, bits);
    while (true) {
      const unsigned long long cur = atomicCAS(&table[h], 0ull, entry);
      if (cur == 0ull) break;
      if (static_cast<uint32_t>(cur) == key) {
        atomicAdd(&table[h], 1ull << 32);
        break;
      }
      h = (h + 1) & mask;
    }
  }
}

__global__ void __launch_bounds__(256)
    join_np_probe_kernel(const int32_t *__restrict__ keys, int64_t n,
                         const unsigned long long *__restrict__ table, int bits,
                         unsigned long long *__restrict__ count) {
  __shared__ unsigned long long s_red[8];
  const uint32_t mask = (1u << bits) - 1u;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned long long matches = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t key = static_cast<uint32_t>(__ldg(keys + i));
    uint32_t h = np_slot(key, bits);
    unsigned long long e;
    while ((e = table[h]) != 0ull) {  // plain loads: random reads are slower on the .nc path
      if (static_cast<uint32_t>(e) == key) {
        matches += e >> 32;
        break;
      }
      h = (h + 1) & mask;
    }
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) matches += __shfl_xor_sync(0xffffffffu, matches, m);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = matches;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < 8; ++w) t += s_red[w];
    if (t) atomicAdd(count, t);
  }
}

int np_bits(int64_t build_len) {
  int bits = 1;
  while ((int64_t{1} << bits) < 2 * build_len) ++bits;  // load factor <= 0.5
  return bits;
}

constexpr int kMaxJoinBuckets = 8192;  // the split's limit

// Partitions of at most half a build chunk of S tuples, up to 8192 of them
// (2^26 uniform S tuples: 8192 partitions of one chunk each, so R's partition
// is probed once).
int auto_buckets(int64_t s_len) {
  int b = 1;
  while (b < kMaxJoinBuckets && s_len / b > kChunk / 2) b *= 2;
  return b;
}

struct JoinLayout {
  size_t r_part, s_part, r_start, s_start, split_ws, bytes;
};

JoinLayout join_layout(int64_t r_len, int64_t s_len, int buckets) {
  JoinLayout L{};
  size_t o = 0;
  auto take = [&](size_t b) {
    const size_t at = o;
    o += round_up(b, 256);
    return at;
  };
  L.r_part = take(4 * static_cast<size_t>(max64(r_len, 1)));
  L.s_part = take(4 * static_cast<size_t>(max64(s_len, 1)));
  L.r_start = take(4 * static_cast<size_t>(buckets));
  L.s_start = take(4 * static_cast<size_t>(buckets));
  const size_t sw = std::max(edpp_split_workspace_size(max64(r_len, 1), buckets, EDPP_KO),
                             edpp_split_workspace_size(max64(s_len, 1), buckets, EDPP_KO));
  L.split_ws = take(sw);
  L.bytes = o;
  return L;
}

}  // namespace
}  // namespace edpp

extern "C" {

size_t edpp_hash_join_workspace_size(int64_t r_len, int64_t s_len, int buckets) {
  if (r_len < 0 || s_len < 0) return 0;
  if (buckets <= 0) buckets = edpp::auto_buckets(s_len);
  if (buckets > edpp::kMaxJoinBuckets || (buckets & (buckets - 1))) return 0;
  return edpp::join_layout(r_len, s_len, buckets).bytes;
}

int edpp_hash_join_count(const int32_t *r_keys, int64_t r_len, const int32_t *s_keys,
                         int64_t s_len, int buckets, unsigned long long *d_count, void *ws,
                         size_t ws_bytes, void *stream) {
  using namespace edpp;
  if (r_len < 0 || s_len < 0 || r_len > INT32_MAX || s_len > INT32_MAX || !d_count)
    return EDPP_EINVAL;
  if (buckets <= 0) buckets = auto_buckets(s_len);
  if (buckets > kMaxJoinBuckets || (buckets & (buckets - 1))) return EDPP_EINVAL;
  cudaStream_t st = as_stream(stream);
  if (cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st) != cudaSuccess) return EDPP_ECUDA;
  if (r_len == 0 || s_len == 0) return EDPP_OK;
  if (!r_keys || !s_keys) return EDPP_EINVAL;
  const JoinLayout L = join_layout(r_len, s_len, buckets);
  if (!ws || ws_bytes < L.bytes) return EDPP_ENOMEM;
  char *w = static_cast<char *>(ws);
  int32_t *rp = reinterpret_cast<int32_t *>(w + L.r_part);
  int32_t *sp = reinterpret_cast<int32_t *>(w + L.s_part);
  int32_t *rs = reinterpret_cast<int32_t *>(w + L.r_start);
  int32_t *ss = reinterpret_cast<int32_t *>(w + L.s_start);
  void *sws = w + L.split_ws;
  const size_t sws_bytes = ws_bytes - L.split_ws;
  int s = edpp_split_i32(r_keys, rp, rs, r_len, buckets, EDPP_KO, nullptr, nullptr, sws, sws_bytes,
                         stream);
  if (s != EDPP_OK) return s;
  s = edpp_split_i32(s_keys, sp, ss, s_len, buckets, EDPP_KO, nullptr, nullptr, sws, sws_bytes,
                     stream);
  if (s != EDPP_OK) return s;
  static std::once_flag once[64];
  static cudaError_t attr[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::call_once(once[dev], [dev] {
    attr[dev] = cudaFuncSetAttribute(join_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(kTable * sizeof(unsigned long long)));
  });
  if (attr[dev] != cudaSuccess) return EDPP_ECUDA;
  join_probe_kernel<<<static_cast<unsigned>(buckets), kThreads, kTable * sizeof(unsigned long long),
                      st>>>(rp, r_len, rs, sp, s_len, ss, buckets, d_count);
  return launch_status();
}

size_t edpp_hash_join_np_workspace_size(int64_t build_len) {
  if (build_len < 0 || build_len > INT32_MAX) return 0;
  return (size_t{1} << edpp::np_bits(edpp::max64(build_len, 1))) * sizeof(unsigned long long);
}

int edpp_hash_join_np_count(const int32_t *build_keys, int64_t build_len, const int32_t *probe_keys,
                            int64_t probe_len, unsigned long long *d_count, void *ws,
                            size_t ws_bytes, void *stream) {
  using namespace edpp;
  if (build_len < 0 || probe_len < 0 || build_len > INT32_MAX || probe_len > INT32_MAX || !d_count)
    return EDPP_EINVAL;
  cudaStream_t st = as_stream(stream);
  if (cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st) != cudaSuccess) return EDPP_ECUDA;
  if (build_len == 0 || probe_len == 0) return EDPP_OK;
  if (!build_keys || !probe_keys) return EDPP_EINVAL;
  const int bits = np_bits(build_len);
  const size_t bytes = (size_t{1} << bits) * sizeof(unsigned long long);
  if (!ws || ws_bytes < bytes || !aligned16(ws)) return EDPP_ENOMEM;
  auto *table = static_cast<unsigned long long *>(ws);
  if (cudaMemsetAsync(table, 0, bytes, st) != cudaSuccess) return EDPP_ECUDA;
  const int sms = device_sm_count();
  const int64_t cap = static_cast<int64_t>(sms) * 8;  // 8 resident blocks of 256 per SM
  const unsigned gb = static_cast<unsigned>(std::max<int64_t>(1, std::min(cap, (build_len + 255) / 256)));
  join_np_build_kernel<<<gb, 256, 0, st>>>(build_keys, build_len, table, bits);
  int s = launch_status();
  if (s != EDPP_OK) return s;
  const unsigned gp = static_cast<unsigned>(std::max<int64_t>(1, std::min(cap, (probe_len + 255) / 256)));
  join_np_probe_kernel<<<gp, 256, 0, st>>>(probe_keys, probe_len, table, bits, d_count);
  return launch_status();
}

}  // extern "C"
