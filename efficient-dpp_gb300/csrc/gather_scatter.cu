// gather_scatter.cu — multi-pass gather and scatter of int32 payloads.
//
// Semantics follow the reference's OpenCL primitives:
//   gather : out[i] = in[loc[i]]           (opencl/kernels/gather_kernel.cl:6-21)
//   scatter: out[loc[i]] = in[i]           (opencl/kernels/scatter_kernel.cl:6-22)
// split into `pass` launches, pass k serving only indices in the window
// [k*ceil(n/pass), (k+1)*ceil(n/pass)) so that the random side of the
// access stays within a slice of the array that can live in L2
// (opencl/primitives/gatherImpl.cpp:38-53, scatterImpl.cpp:39-52).  Every
// pass reads the whole index array, as in the reference.  The last window is
// clamped to n, so an index outside [0,n) is skipped in every pass (the
// reference would read or write past the array there); for every valid
// index the result is the reference's.
//
// GB300 form: each thread takes 16-byte vectors of loc (4 indices) with
// kUnroll vectors per step, issues all random loads of a step before any
// store (gather) or all streaming loads before the random stores (scatter),
// and writes gathered vectors back as 128-bit streaming stores when all four
// lanes fall inside the window.
#include "common.cuh"

namespace edpp {
namespace {

constexpr int kThreads = 256;
constexpr int kUnroll = 4;

__device__ __forceinline__ bool in_window(int32_t p, int32_t from, int32_t span) {
  return static_cast<uint32_t>(p - from) < static_cast<uint32_t>(span);
}

// Random read of the gathered payload: a plain global load.  (The read-only
// path, ld.global.nc, measured much slower for random 4-byte reads on GB300:
// 2^26 single pass 1.21 against 1.03 ms, 16 passes 2.27 against 1.52 ms.)
__device__ __forceinline__ int32_t ld_random(const int32_t *p) { return *p; }

// U vectors of 4 indices at vector positions i, i+stride, ..., i+(U-1)*stride.
template <bool kScatter, int U>
__device__ __forceinline__ void pass_step(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                          const int32_t *__restrict__ loc, int64_t i,
                                          int64_t stride, int32_t from, int32_t span) {
  const int4 *loc4 = reinterpret_cast<const int4 *>(loc);
  int4 l[U];
#pragma unroll
  for (int u = 0; u < U; ++u) l[u] = __ldcs(loc4 + i + u * stride);
  if (!kScatter) {
    int4 *out4 = reinterpret_cast<int4 *>(out);
    int4 v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      v[u].x = in_window(l[u].x, from, span) ? ld_random(in + l[u].x) : 0;
      v[u].y = in_window(l[u].y, from, span) ? ld_random(in + l[u].y) : 0;
      v[u].z = in_window(l[u].z, from, span) ? ld_random(in + l[u].z) : 0;
      v[u].w = in_window(l[u].w, from, span) ? ld_random(in + l[u].w) : 0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t j = i + u * stride;
      const bool a = in_window(l[u].x, from, span), b = in_window(l[u].y, from, span),
                 c = in_window(l[u].z, from, span), d = in_window(l[u].w, from, span);
      if (a && b && c && d) {
        __stcs(out4 + j, v[u]);
      } else {
        int32_t *o = out + 4 * j;
        if (a) o[0] = v[u].x;
        if (b) o[1] = v[u].y;
        if (c) o[2] = v[u].z;
        if (d) o[3] = v[u].w;
      }
    }
  } else {
    const int4 *in4 = reinterpret_cast<const int4 *>(in);
    int4 v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) v[u] = __ldcs(in4 + i + u * stride);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (in_window(l[u].x, from, span)) out[l[u].x] = v[u].x;
      if (in_window(l[u].y, from, span)) out[l[u].y] = v[u].y;
      if (in_window(l[u].z, from, span)) out[l[u].z] = v[u].z;
      if (in_window(l[u].w, from, span)) out[l[u].w] = v[u].w;
    }
  }
}

template <bool kScatter, int U>
__global__ void __launch_bounds__(kThreads)
    pass_vec_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                    const int32_t *__restrict__ loc, int64_t n, int32_t from, int32_t span) {
  const int64_t n4 = n >> 2;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * kThreads;
  int64_t i = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x;
  for (; i + (U - 1) * stride < n4; i += U * stride)
    pass_step<kScatter, U>(in, out, loc, i, stride, from, span);
  for (; i < n4; i += stride) pass_step<kScatter, 1>(in, out, loc, i, stride, from, span);
  // Scalar tail [4*n4, n).
  if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {
    const int64_t k = 4 * n4 + threadIdx.x;
    const int32_t p = loc[k];
    if (in_window(p, from, span)) {
      if (kScatter) out[p] = in[k];
      else out[k] = in[p];
    }
  }
}

template <bool kScatter>
__global__ void __launch_bounds__(kThreads)
    pass_scalar_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                       const int32_t *__restrict__ loc, int64_t n, int32_t from, int32_t span) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * kThreads;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x; k < n; k += stride) {
    const int32_t p = loc[k];
    if (in_window(p, from, span)) {
      if (kScatter) out[p] = in[k];
      else out[k] = in[p];
    }
  }
}

template <bool kScatter>
int multipass(const int32_t *in, int32_t *out, int64_t n, const int32_t *loc, int pass,
              void *stream) {
  if (n < 0 || pass < 1) return EDPP_EINVAL;
  if (n == 0) return EDPP_OK;
  if (!in || !out || !loc) return EDPP_EINVAL;
  if (n > INT32_MAX) return EDPP_EINVAL;  // int32 indices address at most 2^31-1 elements
  cudaStream_t st = as_stream(stream);
  const bool vec = aligned16(loc) && aligned16(out) && (!kScatter || aligned16(in));
  // One pass (every index in window): one 4-index vector per thread over a
  // grid covering the array.  Several passes (most indices skipped): a grid
  // of 16 blocks of 256 threads per SM, kUnroll vectors in flight per thread.
  // Measured on GB300, 2^26 / 2^28 gathers: one pass 1.03 / 5.66 ms with the
  // unrolled form, 1.00 / 5.34 ms with the covering grid; 16 passes 1.52 /
  // 7.37 ms unrolled, 1.56 / 7.83 ms covering.
  const bool cover = pass == 1;
  const int64_t per_block = static_cast<int64_t>(kThreads) * 4 * (cover ? 1 : kUnroll);
  int64_t blocks = (n + per_block - 1) / per_block;
  const int64_t cap = cover ? int64_t{INT32_MAX} : static_cast<int64_t>(device_sm_count()) * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  // Window arithmetic of gatherImpl.cpp:38-44 (len_per_run = ceil(n/pass)).
  const int64_t len_per_run = (n + pass - 1) / pass;
  for (int k = 0; k < pass; ++k) {
    const int64_t from = static_cast<int64_t>(k) * len_per_run;
    if (from >= n) break;  // windows past the end serve no valid index
    const int64_t to = min64(n, from + len_per_run);
    const int32_t f = static_cast<int32_t>(from), span = static_cast<int32_t>(to - from);
    if (vec && cover)
      pass_vec_kernel<kScatter, 1><<<static_cast<unsigned>(blocks), kThreads, 0, st>>>(
          in, out, loc, n, f, span);
    else if (vec)
      pass_vec_kernel<kScatter, kUnroll><<<static_cast<unsigned>(blocks), kThreads, 0, st>>>(
          in, out, loc, n, f, span);
    else
      pass_scalar_kernel<kScatter><<<static_cast<unsigned>(blocks), kThreads, 0, st>>>(in, out, loc,
                                                                                      n, f, span);
    const int s = launch_status();
    if (s != EDPP_OK) return s;
  }
  return EDPP_OK;
}

}  // namespace
}  // namespace edpp

extern "C" {

int edpp_gather_i32(const int32_t *in, int32_t *out, int64_t length, const int32_t *loc, int pass,
                    void *stream) {
  return edpp::multipass<false>(in, out, length, loc, pass, stream);
}

int edpp_scatter_i32(const int32_t *in, int32_t *out, int64_t length, const int32_t *loc, int pass,
                     void *stream) {
  return edpp::multipass<true>(in, out, length, loc, pass, stream);
}

}  // extern "C"
