// ref_cuda_runner.cu — launches the reference's own CUDA kernels.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles the reference's
// cuda/test_{split,gather,scatter,bandwidth}.cu device code, unchanged, into
// oracle/_ref/*.cubin; this runner loads those modules with the driver API
// and replays the host sequence of each reference test on caller arrays:
//   split:    pre_scan<<<n/256,256>>> -> cub::DeviceScan::ExclusiveSum over
//             buckets*num_warps -> post_scan<<<n/256,256>>>
//             (cuda/test_split.cu:149-186)
//   gather / scatter: gather_kernel / scatter_kernel<<<ceil(n/256),256>>>
//             (cuda/test_gather.cu:23-24,46; cuda/test_scatter.cu)
//   stream:   copy/scale/addition/triad_kernel<<<ceil(n/256),256>>>
//             (cuda/test_bandwidth.cu:47-107)
//   scan:     cub::DeviceScan::ExclusiveSum, the call of cuda/test_scan.cu:45-47
// Inputs are host arrays; every precondition the reference kernels rely on
// (n a multiple of 256 for split, keys < buckets, indices in range) is checked
// on the host before anything is launched, so the reference kernels never
// run outside their bounds.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cub/cub.cuh>
#include <cstdint>
#include <cstdio>
#include <string>

namespace {

CUmodule g_mod[4];
bool g_loaded = false;
enum { kSplit = 0, kGather = 1, kScatter = 2, kBandwidth = 3 };

int load(const char *dir) {
  if (g_loaded) return 0;
  if (cudaFree(nullptr) != cudaSuccess) return 1;  // primary context
  const char *names[4] = {"test_split", "test_gather", "test_scatter", "test_bandwidth"};
  for (int i = 0; i < 4; ++i) {
    const std::string p = std::string(dir) + "/" + names[i] + ".cubin";
    if (cuModuleLoad(&g_mod[i], p.c_str()) != CUDA_SUCCESS) return 2;
  }
  g_loaded = true;
  return 0;
}

int launch(int mod, const char *name, unsigned grid, void **args) {
  CUfunction f;
  if (cuModuleGetFunction(&f, g_mod[mod], name) != CUDA_SUCCESS) return 3;
  if (cuLaunchKernel(f, grid, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr) != CUDA_SUCCESS) return 4;
  if (cudaDeviceSynchronize() != cudaSuccess) return 5;
  return 0;
}

template <typename T> struct Dev {
  T *p = nullptr;
  explicit Dev(size_t n) {
    if (cudaMalloc(&p, n * sizeof(T) + 16) != cudaSuccess) p = nullptr;
  }
  ~Dev() {
    if (p) cudaFree(p);
  }
};

}  // namespace

extern "C" {

int refcu_init(const char *cubin_dir) { return load(cubin_dir); }

// Stable key-only split of the CUDA reference; keys must be < 2^bucket_bits.
int refcu_split(const int *h_keys, int *h_out, long long n, int bucket_bits) {
  if (!g_loaded) return 10;
  if (n <= 0 || n % 256 != 0 || bucket_bits < 1 || bucket_bits > 8) return 11;
  const int buckets = 1 << bucket_bits;
  for (long long i = 0; i < n; ++i)
    if (h_keys[i] < 0 || h_keys[i] >= buckets) return 12;
  const long long grid = n / 256, num_warps = grid * 256 / 32;
  if (buckets * num_warps >= (1ll << 31)) return 13;  // int indexing of the reference
  Dev<int> k_in(n), k_out(n), his(buckets * num_warps), his_s(buckets * num_warps);
  if (!k_in.p || !k_out.p || !his.p || !his_s.p) return 14;
  cudaMemcpy(k_in.p, h_keys, n * sizeof(int), cudaMemcpyHostToDevice);
  int len = static_cast<int>(n);
  void *a1[] = {&k_in.p, &his.p, &len, &bucket_bits};
  if (int e = launch(kSplit, "_Z8pre_scanPiS_ii", static_cast<unsigned>(grid), a1)) return e;
  void *tmp = nullptr;
  size_t tmp_bytes = 0;
  const int m = static_cast<int>(buckets * num_warps);
  cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, his.p, his_s.p, m);
  if (cudaMalloc(&tmp, tmp_bytes) != cudaSuccess) return 14;
  cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, his.p, his_s.p, m);
  cudaDeviceSynchronize();
  cudaFree(tmp);
  void *a2[] = {&k_in.p, &k_out.p, &his_s.p, &len, &bucket_bits};
  if (int e = launch(kSplit, "_Z9post_scanPiS_S_ii", static_cast<unsigned>(grid), a2)) return e;
  cudaMemcpy(h_out, k_out.p, n * sizeof(int), cudaMemcpyDeviceToHost);
  return cudaGetLastError() == cudaSuccess ? 0 : 15;
}

// gather (scatter=0) or scatter (scatter=1) of the CUDA reference.
int refcu_gather_scatter(int scatter, const int *h_in, int *h_out, const int *h_idx, long long n) {
  if (!g_loaded) return 10;
  if (n <= 0 || n >= (1ll << 31)) return 11;
  for (long long i = 0; i < n; ++i)
    if (h_idx[i] < 0 || h_idx[i] >= n) return 12;
  Dev<int> in(n), out(n), idx(n);
  if (!in.p || !out.p || !idx.p) return 14;
  cudaMemcpy(in.p, h_in, n * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(idx.p, h_idx, n * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(out.p, h_out, n * sizeof(int), cudaMemcpyHostToDevice);
  int len = static_cast<int>(n);
  void *args[] = {&in.p, &out.p, &idx.p, &len};
  const unsigned grid = static_cast<unsigned>((n + 255) / 256);
  int e = scatter ? launch(kScatter, "_Z14scatter_kernelPiS_S_i", grid, args)
                  : launch(kGather, "_Z13gather_kernelPiS_S_i", grid, args);
  if (e) return e;
  cudaMemcpy(h_out, out.p, n * sizeof(int), cudaMemcpyDeviceToHost);
  return cudaGetLastError() == cudaSuccess ? 0 : 15;
}

// op: 0 copy, 1 scale(x3), 2 addition, 3 triad (a + 3b), int32.
int refcu_stream_i32(int op, const int *h_a, const int *h_b, int *h_c, long long n) {
  if (!g_loaded) return 10;
  if (n <= 0 || n >= (1ll << 31) || op < 0 || op > 3) return 11;
  Dev<int> a(n), b(n), c(n);
  if (!a.p || !b.p || !c.p) return 14;
  cudaMemcpy(a.p, h_a, n * sizeof(int), cudaMemcpyHostToDevice);
  if (op >= 2) cudaMemcpy(b.p, h_b, n * sizeof(int), cudaMemcpyHostToDevice);
  int len = static_cast<int>(n);
  const unsigned grid = static_cast<unsigned>((n + 255) / 256);
  int e;
  if (op == 0) {
    void *args[] = {&a.p, &c.p, &len};
    e = launch(kBandwidth, "_Z11copy_kernelPiS_i", grid, args);
  } else if (op == 1) {
    void *args[] = {&a.p, &c.p, &len};
    e = launch(kBandwidth, "_Z12scale_kernelPiS_i", grid, args);
  } else {
    void *args[] = {&a.p, &b.p, &c.p, &len};
    e = launch(kBandwidth, op == 2 ? "_Z15addition_kernelPiS_S_i" : "_Z12triad_kernelPiS_S_i",
               grid, args);
  }
  if (e) return e;
  cudaMemcpy(h_c, c.p, n * sizeof(int), cudaMemcpyDeviceToHost);
  return cudaGetLastError() == cudaSuccess ? 0 : 15;
}

// cub::DeviceScan::ExclusiveSum on int32, as cuda/test_scan.cu:45-47 calls it.
int refcu_cub_exclusive_sum_i32(const int *h_in, int *h_out, long long n) {
  if (n <= 0 || n >= (1ll << 31)) return 11;
  if (cudaFree(nullptr) != cudaSuccess) return 1;
  Dev<int> in(n), out(n);
  if (!in.p || !out.p) return 14;
  cudaMemcpy(in.p, h_in, n * sizeof(int), cudaMemcpyHostToDevice);
  void *tmp = nullptr;
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in.p, out.p, static_cast<int>(n));
  if (cudaMalloc(&tmp, tmp_bytes) != cudaSuccess) return 14;
  cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in.p, out.p, static_cast<int>(n));
  cudaDeviceSynchronize();
  cudaFree(tmp);
  cudaMemcpy(h_out, out.p, n * sizeof(int), cudaMemcpyDeviceToHost);
  return cudaGetLastError() == cudaSuccess ? 0 : 15;
}

// ---- timing of the reference kernels (device-resident data, CUDA events) ----
// Each returns 0 and *ms = mean milliseconds per call over `reps` calls after
// one warm-up call; inputs are checked on the host exactly as above.
}  // extern "C"

namespace {
template <typename F> int time_reps(int reps, F &&call, float *ms) {
  if (int e = call()) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a);
  for (int r = 0; r < reps; ++r)
    if (int e = call()) return e;
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  cudaEventElapsedTime(ms, a, b);
  *ms /= reps;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return cudaGetLastError() == cudaSuccess ? 0 : 15;
}

int launch_async(int mod, const char *name, unsigned grid, void **args) {
  CUfunction f;
  if (cuModuleGetFunction(&f, g_mod[mod], name) != CUDA_SUCCESS) return 3;
  return cuLaunchKernel(f, grid, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr) == CUDA_SUCCESS ? 0 : 4;
}
}  // namespace

extern "C" {

int refcu_time_gather_scatter(int scatter, const int *h_idx, long long n, int reps, float *ms) {
  if (!g_loaded) return 10;
  if (n <= 0 || n >= (1ll << 31) || reps < 1) return 11;
  for (long long i = 0; i < n; ++i)
    if (h_idx[i] < 0 || h_idx[i] >= n) return 12;
  Dev<int> in(n), out(n), idx(n);
  if (!in.p || !out.p || !idx.p) return 14;
  cudaMemset(in.p, 0, n * sizeof(int));
  cudaMemcpy(idx.p, h_idx, n * sizeof(int), cudaMemcpyHostToDevice);
  int len = static_cast<int>(n);
  void *args[] = {&in.p, &out.p, &idx.p, &len};
  const unsigned grid = static_cast<unsigned>((n + 255) / 256);
  return time_reps(reps, [&] {
    return scatter ? launch_async(kScatter, "_Z14scatter_kernelPiS_S_i", grid, args)
                   : launch_async(kGather, "_Z13gather_kernelPiS_S_i", grid, args);
  }, ms);
}

int refcu_time_cub_scan(long long n, int reps, float *ms) {
  if (n <= 0 || n >= (1ll << 31) || reps < 1) return 11;
  if (cudaFree(nullptr) != cudaSuccess) return 1;
  Dev<int> in(n), out(n);
  if (!in.p || !out.p) return 14;
  cudaMemset(in.p, 0, n * sizeof(int));
  void *tmp = nullptr;
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in.p, out.p, static_cast<int>(n));
  if (cudaMalloc(&tmp, tmp_bytes) != cudaSuccess) return 14;
  const int e = time_reps(reps, [&] {
    return cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in.p, out.p, static_cast<int>(n)) ==
                   cudaSuccess ? 0 : 4;
  }, ms);
  cudaFree(tmp);
  return e;
}

int refcu_time_split(const int *h_keys, long long n, int bucket_bits, int reps, float *ms) {
  if (!g_loaded) return 10;
  if (n <= 0 || n % 256 != 0 || bucket_bits < 1 || bucket_bits > 8 || reps < 1) return 11;
  const int buckets = 1 << bucket_bits;
  for (long long i = 0; i < n; ++i)
    if (h_keys[i] < 0 || h_keys[i] >= buckets) return 12;
  const long long grid = n / 256, num_warps = grid * 256 / 32;
  if (buckets * num_warps >= (1ll << 31)) return 13;
  Dev<int> k_in(n), k_out(n), his(buckets * num_warps), his_s(buckets * num_warps);
  if (!k_in.p || !k_out.p || !his.p || !his_s.p) return 14;
  cudaMemcpy(k_in.p, h_keys, n * sizeof(int), cudaMemcpyHostToDevice);
  int len = static_cast<int>(n);
  const int m = static_cast<int>(buckets * num_warps);
  void *tmp = nullptr;
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, his.p, his_s.p, m);
  if (cudaMalloc(&tmp, tmp_bytes) != cudaSuccess) return 14;
  void *a1[] = {&k_in.p, &his.p, &len, &bucket_bits};
  void *a2[] = {&k_in.p, &k_out.p, &his_s.p, &len, &bucket_bits};
  const int e = time_reps(reps, [&] {
    if (int r = launch_async(kSplit, "_Z8pre_scanPiS_ii", static_cast<unsigned>(grid), a1)) return r;
    if (cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, his.p, his_s.p, m) != cudaSuccess) return 4;
    return launch_async(kSplit, "_Z9post_scanPiS_S_ii", static_cast<unsigned>(grid), a2);
  }, ms);
  cudaFree(tmp);
  return e;
}

int refcu_time_stream_i32(int op, long long n, int reps, float *ms) {
  if (!g_loaded) return 10;
  if (n <= 0 || n >= (1ll << 31) || op < 0 || op > 3 || reps < 1) return 11;
  Dev<int> a(n), b(n), c(n);
  if (!a.p || !b.p || !c.p) return 14;
  cudaMemset(a.p, 0, n * sizeof(int));
  cudaMemset(b.p, 0, n * sizeof(int));
  int len = static_cast<int>(n);
  const unsigned grid = static_cast<unsigned>((n + 255) / 256);
  void *a2[] = {&a.p, &c.p, &len};
  void *a3[] = {&a.p, &b.p, &c.p, &len};
  static const char *names[4] = {"_Z11copy_kernelPiS_i", "_Z12scale_kernelPiS_i",
                                 "_Z15addition_kernelPiS_S_i", "_Z12triad_kernelPiS_S_i"};
  return time_reps(reps, [&] { return launch_async(kBandwidth, names[op], grid, op < 2 ? a2 : a3); },
                   ms);
}

}  // extern "C"
