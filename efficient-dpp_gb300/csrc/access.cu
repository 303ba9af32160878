// access.cu — memory access-pattern and single-block scan microbenchmarks.
//
// Kernels that measure how the access pattern, the order in which blocks
// visit memory and the per-thread tile size set the bandwidth of the
// primitives; they back the coalescing and tile-size choices of the scan,
// split and gather/scatter kernels with numbers.
//
//   scale (column / row / mixed)  opencl/kernels/mem_kernel.cl:33-69,
//                                 driven by opencl/test/test_access.cpp
//   scale (vector)                GB300 form: 16-byte grid-stride loop
//   block-order sweep (wg_access) mem_kernel.cl:71-87, opencl/test/test_access_wg.cpp
//   cache heat                    mem_kernel.cl:89-107
//   single-block matrix scan      opencl/kernels/scan_local_kernel.cl:530-695,
//                                 driven by opencl/test/test_scan_local.cpp
//
// Index arithmetic is 64-bit (the reference's int indices wrap above 2^31
// elements); the touched index sets are those of the reference kernels.
#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace edpp {
namespace {

constexpr int32_t kScalar = 3;  // SCALAR of the reference's scale kernels

// column-major: thread g touches g, g+G, g+2G, ... (coalesced per step)
__global__ void scale_column_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                    int repeat) {
  const int64_t G = static_cast<int64_t>(gridDim.x) * blockDim.x;
  int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  for (int i = 0; i < repeat; ++i, g += G) out[g] = in[g] * kScalar;
}

// row-major: thread g touches g*repeat .. g*repeat+repeat-1 (strided per step)
__global__ void scale_row_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                 int repeat) {
  const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t begin = g * repeat;
  for (int i = 0; i < repeat; ++i) out[begin + i] = in[begin + i] * kScalar;
}

// mixed: warp w owns [32*repeat*w, 32*repeat*(w+1)), lanes step by 32
__global__ void scale_mixed_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                   int repeat) {
  const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  int64_t idx = 32 * static_cast<int64_t>(repeat) * (g >> 5) + (g & 31);
  for (int i = 0; i < repeat; ++i, idx += 32) out[idx] = in[idx] * kScalar;
}

// vector: 16-byte grid-stride loop over the same n elements, four vectors
// in flight per thread before the stores (the STREAM kernels' shape),
// scalar tail
__global__ void scale_vec_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                 int64_t n) {
  constexpr int kU = 4;
  const int64_t G = static_cast<int64_t>(gridDim.x) * blockDim.x;
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t nv = n >> 2;
  const int4 *vi = reinterpret_cast<const int4 *>(in);
  int4 *vo = reinterpret_cast<int4 *>(out);
  auto scale4 = [](int4 v) {
    v.x *= kScalar;
    v.y *= kScalar;
    v.z *= kScalar;
    v.w *= kScalar;
    return v;
  };
  for (; i + (kU - 1) * G < nv; i += kU * G) {
    int4 v[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) v[u] = __ldcs(vi + i + u * G);
#pragma unroll
    for (int u = 0; u < kU; ++u) __stcs(vo + i + u * G, scale4(v[u]));
  }
  for (; i < nv; i += G) __stcs(vo + i, scale4(__ldcs(vi + i)));
  const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  for (int64_t j = (nv << 2) + g; j < n; j += G) out[j] = in[j] * kScalar;
}

// Block b takes ticket t (atomic), visits chunk order[t] of `len / blocks`
// elements and sums their low bits; out[chunk] gets the sum (the reference
// writes every sum to one word; one word per chunk makes the result checkable).
__global__ void access_wg_kernel(const int32_t *__restrict__ in, int64_t chunk_len,
                                 const int32_t *__restrict__ order, unsigned *ticket,
                                 long long *__restrict__ out) {
  __shared__ int s_w;
  __shared__ long long s_red[32];
  if (threadIdx.x == 0) s_w = order[atomicAdd(ticket, 1u)];
  __syncthreads();
  const int64_t w = s_w;
  const int64_t begin = w * chunk_len, end = begin + chunk_len;
  long long acc = 0;
  for (int64_t c = begin + threadIdx.x; c < end; c += blockDim.x) acc += in[c] & 1;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) s_red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t = 0;
    for (int i = 0; i < static_cast<int>((blockDim.x + 31) >> 5); ++i) t += s_red[i];
    out[w] = t;
  }
}

// write-only warm-up: warp v writes data[c] = c over its warp-chunk
__global__ void cache_heat_kernel(int32_t *__restrict__ data, int64_t length) {
  const int64_t G = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t per = (length + G - 1) / G;
  const int64_t begin = (g >> 5) * 32 * per;
  const int64_t end = min64(length, ((g >> 5) + 1) * 32 * per);
  for (int64_t c = begin + (g & 31); c < end; c += 32) data[c] = static_cast<int32_t>(c);
}

// ---- single-block exclusive scan of 512 * tile elements -------------------
constexpr int kScanThreads = 512;
constexpr int kMaxTile = 49;  // the reference sweeps 1..49 elements per thread

__device__ __forceinline__ void block_scan_serial(int *lsum) {
  // one thread scans the per-thread sums (the reference's local scheme)
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int i = 0; i < kScanThreads; ++i) {
      const int t = lsum[i];
      lsum[i] = acc;
      acc += t;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ int block_scan_warp(int v, int *wsum) {
  // exclusive block scan of one value per thread with warp shuffles
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int s = lane < kScanThreads / 32 ? wsum[lane] : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, d);
      if (lane >= d) s += y;
    }
    if (lane < kScanThreads / 32) wsum[lane] = s;
  }
  __syncthreads();
  return x - v + (warp ? wsum[warp - 1] : 0);
}

// scheme 0 (LM): tile staged in shared memory with coalesced loads; each
// thread reduces and rescans its row of `tile` elements; serial block scan
__global__ void __launch_bounds__(kScanThreads)
    matrix_scan_lm_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out, int tile) {
  extern __shared__ int ldata[];
  __shared__ int lsum[kScanThreads];
  const int total = kScanThreads * tile;
  for (int i = threadIdx.x; i < total; i += kScanThreads) ldata[i] = in[i];
  __syncthreads();
  const int begin = threadIdx.x * tile;
  int acc = 0;
  for (int i = 0; i < tile; ++i) acc += ldata[begin + i];
  lsum[threadIdx.x] = acc;
  block_scan_serial(lsum);
  acc = lsum[threadIdx.x];
  for (int i = 0; i < tile; ++i) {
    const int v = ldata[begin + i];
    ldata[begin + i] = acc;
    acc += v;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < total; i += kScanThreads) out[i] = ldata[i];
}

// scheme 1 (REG): each thread loads its row straight into registers
// (strided across the warp) and writes it back the same way
__global__ void __launch_bounds__(kScanThreads)
    matrix_scan_reg_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out, int tile) {
  __shared__ int lsum[kScanThreads];
  int reg[kMaxTile];
  const int64_t offset = static_cast<int64_t>(threadIdx.x) * tile;
  int acc = 0;
#pragma unroll
  for (int i = 0; i < kMaxTile; ++i)
    if (i < tile) {
      reg[i] = in[offset + i];
      acc += reg[i];
    }
  lsum[threadIdx.x] = acc;
  block_scan_serial(lsum);
  acc = lsum[threadIdx.x];
#pragma unroll
  for (int i = 0; i < kMaxTile; ++i)
    if (i < tile) {
      out[offset + i] = acc;
      acc += reg[i];
    }
}

// scheme 2 (LM_REG): coalesced loads into shared memory, rows moved to
// registers, results written back through shared memory
__global__ void __launch_bounds__(kScanThreads)
    matrix_scan_lm_reg_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out, int tile) {
  extern __shared__ int ldata[];
  __shared__ int lsum[kScanThreads];
  const int total = kScanThreads * tile;
  for (int i = threadIdx.x; i < total; i += kScanThreads) ldata[i] = in[i];
  __syncthreads();
  int reg[kMaxTile];
  const int begin = threadIdx.x * tile;
  int acc = 0;
#pragma unroll
  for (int i = 0; i < kMaxTile; ++i)
    if (i < tile) {
      reg[i] = ldata[begin + i];
      acc += reg[i];
    }
  lsum[threadIdx.x] = acc;
  block_scan_serial(lsum);
  acc = lsum[threadIdx.x];
#pragma unroll
  for (int i = 0; i < kMaxTile; ++i)
    if (i < tile) {
      ldata[begin + i] = acc;
      acc += reg[i];
    }
  __syncthreads();
  for (int i = threadIdx.x; i < total; i += kScanThreads) out[i] = ldata[i];
}

// scheme 3 (WARP, GB300 form): LM_REG with the serial block scan replaced by
// a two-level warp-shuffle scan
__global__ void __launch_bounds__(kScanThreads)
    matrix_scan_warp_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out, int tile) {
  extern __shared__ int ldata[];
  __shared__ int wsum[kScanThreads / 32];
  const int total = kScanThreads * tile;
  for (int i = threadIdx.x; i < total; i += kScanThreads) ldata[i] = in[i];
  __syncthreads();
  int reg[kMaxTile];
  const int begin = threadIdx.x * tile;
  int acc = 0;
#pragma unroll
  for (int i = 0; i < kMaxTile; ++i)
    if (i < tile) {
      reg[i] = ldata[begin + i];
      acc += reg[i];
    }
  acc = block_scan_warp(acc, wsum);
#pragma unroll
  for (int i = 0; i < kMaxTile; ++i)
    if (i < tile) {
      ldata[begin + i] = acc;
      acc += reg[i];
    }
  __syncthreads();
  for (int i = threadIdx.x; i < total; i += kScanThreads) out[i] = ldata[i];
}

int set_smem_once(const void *fn, int bytes) {
  static std::mutex mu;
  static int done_bytes[4][64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  const int k = fn == reinterpret_cast<const void *>(matrix_scan_lm_kernel)       ? 0
                : fn == reinterpret_cast<const void *>(matrix_scan_lm_reg_kernel) ? 1
                                                                                  : 2;
  std::lock_guard<std::mutex> lock(mu);
  if (done_bytes[k][dev] >= bytes) return EDPP_OK;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
    return EDPP_ECUDA;
  done_bytes[k][dev] = bytes;
  return EDPP_OK;
}

}  // namespace
}  // namespace edpp

extern "C" {

int edpp_access_scale_i32(const int32_t *in, int32_t *out, int repeat, int pattern, int local_size,
                          int grid_size, void *stream) {
  using namespace edpp;
  if (repeat < 0 || local_size <= 0 || local_size > 1024 || grid_size <= 0 || !in || !out)
    return EDPP_EINVAL;
  if (repeat == 0) return EDPP_OK;
  const int64_t threads = static_cast<int64_t>(local_size) * grid_size;
  cudaStream_t st = as_stream(stream);
  switch (pattern) {
    case EDPP_ACCESS_COLUMN:
      scale_column_kernel<<<grid_size, local_size, 0, st>>>(in, out, repeat);
      break;
    case EDPP_ACCESS_ROW:
      scale_row_kernel<<<grid_size, local_size, 0, st>>>(in, out, repeat);
      break;
    case EDPP_ACCESS_MIXED:
      if (threads % 32) return EDPP_EINVAL;  // warps must tile the index range
      scale_mixed_kernel<<<grid_size, local_size, 0, st>>>(in, out, repeat);
      break;
    case EDPP_ACCESS_VEC: {
      if (!aligned16(in) || !aligned16(out)) return EDPP_EINVAL;
      const int64_t n = threads * repeat;
      const int64_t cap = static_cast<int64_t>(device_sm_count()) * 8;  // 8 blocks of 256 per SM
      const unsigned g = static_cast<unsigned>(std::max<int64_t>(1, std::min(cap, (n / 4 + 255) / 256)));
      scale_vec_kernel<<<g, 256, 0, st>>>(in, out, n);
      break;
    }
    default:
      return EDPP_EINVAL;
  }
  return launch_status();
}

int edpp_access_wg_i32(const int32_t *in, int64_t len, const int32_t *order, int grid_size,
                       int local_size, unsigned *ticket, long long *out, void *stream) {
  using namespace edpp;
  if (!in || !order || !ticket || !out || grid_size <= 0 || local_size <= 0 || local_size > 1024 ||
      len < grid_size)
    return EDPP_EINVAL;
  cudaStream_t st = as_stream(stream);
  if (cudaMemsetAsync(ticket, 0, sizeof(unsigned), st) != cudaSuccess) return EDPP_ECUDA;
  access_wg_kernel<<<grid_size, local_size, 0, st>>>(in, len / grid_size, order, ticket, out);
  return launch_status();
}

int edpp_cache_heat_i32(int32_t *data, int64_t length, int local_size, int grid_size, void *stream) {
  using namespace edpp;
  if (!data || length < 0 || local_size <= 0 || local_size > 1024 || grid_size <= 0)
    return EDPP_EINVAL;
  if (length == 0) return EDPP_OK;
  cache_heat_kernel<<<grid_size, local_size, 0, as_stream(stream)>>>(data, length);
  return launch_status();
}

int edpp_local_scan_i32(const int32_t *in, int32_t *out, int tile_size, int scheme, int repeat,
                        void *stream) {
  using namespace edpp;
  if (!in || !out || tile_size < 1 || tile_size > kMaxTile || repeat < 0) return EDPP_EINVAL;
  if (in == out) return EDPP_EINVAL;  // the register scheme writes before all rows are read
  cudaStream_t st = as_stream(stream);
  const int smem = kScanThreads * tile_size * static_cast<int>(sizeof(int));
  const void *fn = nullptr;
  switch (scheme) {
    case EDPP_LOCAL_SCAN_LM: fn = reinterpret_cast<const void *>(matrix_scan_lm_kernel); break;
    case EDPP_LOCAL_SCAN_REG: fn = nullptr; break;
    case EDPP_LOCAL_SCAN_LM_REG: fn = reinterpret_cast<const void *>(matrix_scan_lm_reg_kernel); break;
    case EDPP_LOCAL_SCAN_WARP: fn = reinterpret_cast<const void *>(matrix_scan_warp_kernel); break;
    default: return EDPP_EINVAL;
  }
  if (fn) {
    const int s = set_smem_once(fn, smem);
    if (s != EDPP_OK) return s;
  }
  for (int r = 0; r < repeat; ++r) {
    switch (scheme) {
      case EDPP_LOCAL_SCAN_LM:
        matrix_scan_lm_kernel<<<1, kScanThreads, smem, st>>>(in, out, tile_size);
        break;
      case EDPP_LOCAL_SCAN_REG:
        matrix_scan_reg_kernel<<<1, kScanThreads, 0, st>>>(in, out, tile_size);
        break;
      case EDPP_LOCAL_SCAN_LM_REG:
        matrix_scan_lm_reg_kernel<<<1, kScanThreads, smem, st>>>(in, out, tile_size);
        break;
      default:
        matrix_scan_warp_kernel<<<1, kScanThreads, smem, st>>>(in, out, tile_size);
        break;
    }
    const int s = launch_status();
    if (s != EDPP_OK) return s;
  }
  return EDPP_OK;
}

}  // extern "C"
