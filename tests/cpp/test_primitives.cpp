// test_primitives.cpp — the reference's test drivers, ported onto the GB300
// primitive API (include/edpp_primitives.hpp): same calls, same checks.
//   gather / scatter : opencl/test/test_gather.cpp:41-70, test_scatter.cpp:63-69
//   scan             : opencl/test/test_scan_global.cpp:38-73
//   split            : opencl/test/test_split.cpp:164-203 (plus stability)
// Exit status 0 when every check passes.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <vector>

#include "edpp_primitives.hpp"

using namespace edpp::primitives;

extern "C" void edpp_gen_permutation_i32(int32_t *out, int64_t n, uint64_t seed);
extern "C" void edpp_gen_uniform_i32(int32_t *out, int64_t n, uint64_t seed, int64_t lo, int64_t hi);
extern "C" void edpp_gen_keys_uniform(int32_t *out, int64_t n, uint64_t seed);

static int failures = 0;
#define CHECK(c, ...)                   \
  do {                                  \
    if (!(c)) {                         \
      std::printf("FAIL: " __VA_ARGS__); \
      std::printf("\n");                \
      ++failures;                       \
    }                                   \
  } while (0)

template <typename T> T *dev(const std::vector<T> &h) {
  T *d = nullptr;
  cudaMalloc(&d, h.size() * sizeof(T) + 16);
  cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
  return d;
}
template <typename T> std::vector<T> host(const T *d, size_t n) {
  std::vector<T> h(n);
  cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost);
  return h;
}

static void test_gather_scatter(int len) {
  std::vector<int> h_in(len), h_loc(len);
  for (int i = 0; i < len; ++i) h_in[i] = i;
  edpp_gen_permutation_i32(h_loc.data(), len, 2);
  int *d_in = dev(h_in), *d_loc = dev(h_loc), *d_out = dev(std::vector<int>(len, 0));
  for (int pass = 1; pass <= 32; pass <<= 1) {
    double ms = gather(d_in, d_out, len, d_loc, 1024, len / 1024 / 16 + 1, pass);
    CHECK(ms >= 0, "gather pass=%d returned %f", pass, ms);
    auto h_out = host(d_out, len);
    bool ok = true;
    for (int i = 0; i < len; ++i) ok = ok && h_out[i] == h_in[h_loc[i]];
    CHECK(ok, "gather pass=%d wrong result", pass);
    ms = scatter(d_in, d_out, len, d_loc, 1024, len / 1024 / 16 + 1, pass);
    CHECK(ms >= 0, "scatter pass=%d returned %f", pass, ms);
    h_out = host(d_out, len);
    ok = true;
    for (int i = 0; i < len; ++i) ok = ok && h_out[h_loc[i]] == h_in[i];
    CHECK(ok, "scatter pass=%d wrong result", pass);
  }
  cudaFree(d_in);
  cudaFree(d_loc);
  cudaFree(d_out);
}

static void test_scan(int len) {
  std::vector<int> h_in(len);
  edpp_gen_uniform_i32(h_in.data(), len, 1, 0, 15);  // rand() & 0xf
  int *d_in = dev(h_in), *d_out = dev(std::vector<int>(len, 0));
  for (int algo = 0; algo < 5; ++algo) {
    double ms;
    switch (algo) {
      case 0: ms = scan_RSS(d_in, d_out, len, 1024, 80); break;
      case 1: ms = scan_RSS_single(d_in, d_out, len); break;
      case 2: ms = scan_chained(d_in, d_out, len, 1024, 80, 0, 11); break;
      case 3: ms = scan_SSA(d_in, d_out, len); break;
      default: ms = scan_RTS(d_in, d_out, len); break;
    }
    CHECK(ms >= 0, "scan algo %d returned %f", algo, ms);
    auto h_out = host(d_out, len);
    int acc = 0;
    bool ok = true;
    for (int i = 0; i < len; i++) {
      if (h_out[i] != acc) ok = false;
      acc += h_in[i];
    }
    CHECK(ok, "scan algo %d wrong result (len %d)", algo, len);
  }
  // parameter error of the reference: R == L == 0 returns 1
  CHECK(scan_chained(d_in, d_out, len, 1024, 80, 0, 0) == 1, "scan_chained R=L=0");
  // in place (split runs scan_chained(d_his, d_his, ...))
  double ms = scan_chained(d_in, d_in, len, 64, 39, 112, 0);
  CHECK(ms >= 0, "in-place scan");
  auto h_out = host(d_in, len);
  int acc = 0;
  bool ok = true;
  for (int i = 0; i < len; i++) {
    if (h_out[i] != acc) ok = false;
    acc += h_in[i];
  }
  CHECK(ok, "in-place scan wrong result");
  cudaFree(d_in);
  cudaFree(d_out);
}

static void test_split(int len, int buckets, int algo, DataStruc structure) {
  std::vector<int> h_keys(len), h_vals(len);
  edpp_gen_keys_uniform(h_keys.data(), len, 3);
  for (int i = 0; i < len; ++i) h_vals[i] = i;  // index values make stability visible
  const unsigned mask = buckets - 1;
  std::vector<int> h_in;
  if (structure == KVS_AOS) {
    h_in.resize(2 * len);
    for (int i = 0; i < len; ++i) {
      h_in[2 * i] = h_keys[i];
      h_in[2 * i + 1] = h_vals[i];
    }
  } else {
    h_in = h_keys;
  }
  int *d_in = dev(h_in), *d_out = dev(std::vector<int>(h_in.size(), 0));
  int *d_vin = dev(h_vals), *d_vout = dev(std::vector<int>(len, 0));
  int *d_start = dev(std::vector<int>(buckets, 0));
  const bool soa = structure == KVS_SOA;
  double ms;
  if (algo == 0)
    ms = WI_split(d_in, d_out, d_start, len, buckets, structure, soa ? d_vin : nullptr,
                  soa ? d_vout : nullptr);
  else if (algo == 1)
    ms = WG_split(d_in, d_out, d_start, len, buckets, VARIED_REORDER, structure,
                  soa ? d_vin : nullptr, soa ? d_vout : nullptr);
  else
    ms = single_split(d_in, d_out, len, buckets, true, structure);
  if (algo == 2 && structure == KVS_SOA) {
    CHECK(ms == -1, "single_split must reject SOA");
    return;
  }
  CHECK(ms >= 0, "split algo %d returned %f", algo, ms);
  auto out = host(d_out, h_in.size());
  auto vout = soa ? host(d_vout, len) : std::vector<int>();
  unsigned long in_sum = 0, out_sum = 0;
  int prev = -1, prev_val = -1;
  bool mono = true, stable = true, intact = true;
  for (int i = 0; i < len; ++i) {
    const int k = structure == KVS_AOS ? out[2 * i] : out[i];
    const int v = structure == KVS_AOS ? out[2 * i + 1] : (soa ? vout[i] : -1);
    const int b = k & mask;
    in_sum += h_keys[i] & mask;
    out_sum += b;
    if (b < prev) mono = false;
    if (structure != KO) {
      if (b == prev && v <= prev_val) stable = false;
      if (v < 0 || v >= len || h_keys[v] != k) intact = false;
      prev_val = v;
    }
    prev = b;
  }
  CHECK(mono, "split: buckets not monotone");
  CHECK(in_sum == out_sum, "split: key sum mismatch");
  CHECK(stable, "split: not stable");
  CHECK(intact, "split: values not intact");
  if (algo < 2) {
    auto st = host(d_start, buckets);
    std::vector<int> cnt(buckets, 0);
    for (int i = 0; i < len; ++i) cnt[h_keys[i] & mask]++;
    int acc = 0;
    bool ok = true;
    for (int b = 0; b < buckets; ++b) {
      ok = ok && st[b] == acc;
      acc += cnt[b];
    }
    CHECK(ok, "split: bucket start positions");
  }
  cudaFree(d_in);
  cudaFree(d_out);
  cudaFree(d_vin);
  cudaFree(d_vout);
  cudaFree(d_start);
}

int main() {
  for (int len : {1000, 1 << 20}) test_gather_scatter(len);
  for (int scale = 10; scale <= 24; scale += 7) test_scan(1 << scale);
  test_scan(12345);
  for (int buckets = 2; buckets <= 4096; buckets <<= 3)
    for (int algo = 0; algo < 3; ++algo)
      for (DataStruc s : {KO, KVS_AOS, KVS_SOA}) test_split(100003, buckets, algo, s);
  // reference parameter checks: bucket count not a power of two
  CHECK(WG_split(nullptr, nullptr, nullptr, 10, 3, NO_REORDER, KO) == -1, "buckets=3");
  std::printf("%s (%d failures)\n", failures ? "FAILED" : "PASSED", failures);
  return failures ? 1 : 0;
}
