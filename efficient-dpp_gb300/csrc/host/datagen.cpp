// datagen.cpp — seeded synthetic inputs for benchmarks and the batched /
// served workloads.
//
// All generators draw from splitmix64 (Steele, Lea, Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014): draw i of a stream with
// seed s is mix64(s + (i+1)*0x9E3779B97F4A7C15), so every index can be
// generated independently and the fill is split over host threads with a
// result that does not depend on the thread count.  A bounded draw in
// [0, r) is (x >> 32) * r >> 32 (Lemire's multiply-shift on the high 32
// bits).  The reference's generators are not reproducible
// (random_generator_int depends on the OpenMP schedule,
// openmp/util/utility.cpp:77-85; random_generator_int_unique seeds from
// time(), :90-104), so these replace them.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;

inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

inline uint64_t draw(uint64_t seed, uint64_t i) { return mix64(seed + (i + 1) * kGamma); }

inline uint64_t bounded(uint64_t x, uint64_t r) { return ((x >> 32) * r) >> 32; }

template <typename F> void parallel_for(int64_t n, F f) {
  if (n <= 0) return;
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  if (nt > 64) nt = 64;
  if (n < (1 << 16)) nt = 1;
  const int64_t per = (n + nt - 1) / nt;
  std::vector<std::thread> ts;
  for (unsigned t = 0; t < nt; ++t) {
    const int64_t lo = t * per, hi = std::min<int64_t>(n, lo + per);
    if (lo >= hi) break;
    ts.emplace_back([=] {
      for (int64_t i = lo; i < hi; ++i) f(i);
    });
  }
  for (auto &t : ts) t.join();
}

}  // namespace

extern "C" {

// Draw i of the stream (exposed so other languages can reproduce a fill).
uint64_t edpp_gen_draw(uint64_t seed, uint64_t i) { return draw(seed, i); }

// Integers uniform in [lo, hi] (hi - lo < 2^32).
void edpp_gen_uniform_i32(int32_t *out, int64_t n, uint64_t seed, int64_t lo, int64_t hi) {
  const uint64_t r = static_cast<uint64_t>(hi - lo + 1);
  parallel_for(n, [=](int64_t i) {
    out[i] = static_cast<int32_t>(lo + static_cast<int64_t>(bounded(draw(seed, i), r)));
  });
}

void edpp_gen_uniform_i64(int64_t *out, int64_t n, uint64_t seed, int64_t lo, int64_t hi) {
  const uint64_t r = static_cast<uint64_t>(hi - lo + 1);
  parallel_for(n, [=](int64_t i) {
    out[i] = lo + static_cast<int64_t>(bounded(draw(seed, i), r));
  });
}

// Floats uniform in [lo, hi): 24 random mantissa bits.
void edpp_gen_uniform_f32(float *out, int64_t n, uint64_t seed, float lo, float hi) {
  parallel_for(n, [=](int64_t i) {
    const float u = static_cast<float>(draw(seed, i) >> 40) * (1.0f / 16777216.0f);
    out[i] = lo + u * (hi - lo);
  });
}

// Keys uniform over [0, 2^31).
void edpp_gen_keys_uniform(int32_t *out, int64_t n, uint64_t seed) {
  parallel_for(n, [=](int64_t i) { out[i] = static_cast<int32_t>(draw(seed, i) >> 33); });
}

// Keys whose bucket b = key & (buckets-1) follows Zipf(s): P(b) ~ 1/(b+1)^s,
// with random high bits: key = ((r << log2(buckets)) | b) & 0x7fffffff.
// The bucket uses stream `seed`, the high bits stream `seed ^ 0x5bd1e995`.
void edpp_gen_keys_zipf(int32_t *out, int64_t n, uint64_t seed, int buckets, double s) {
  if (buckets < 1) return;
  int bits = 0;
  while ((1 << bits) < buckets) ++bits;
  std::vector<double> cdf(static_cast<size_t>(buckets));
  double acc = 0.0;
  for (int b = 0; b < buckets; ++b) {
    acc += 1.0 / std::pow(static_cast<double>(b + 1), s);
    cdf[static_cast<size_t>(b)] = acc;
  }
  for (auto &c : cdf) c /= acc;
  cdf.back() = 1.0;
  const double *c = cdf.data();
  const uint64_t seed2 = seed ^ 0x5bd1e995ull;
  parallel_for(n, [=](int64_t i) {
    const double u = static_cast<double>(draw(seed, i) >> 11) * (1.0 / 9007199254740992.0);
    const int b = static_cast<int>(std::upper_bound(c, c + buckets - 1, u) - c);
    const uint32_t r = static_cast<uint32_t>(draw(seed2, i) >> 33);
    out[i] = static_cast<int32_t>(((r << bits) | static_cast<uint32_t>(b)) & 0x7fffffffu);
  });
}

// Uniform random permutation of [0, n) by Fisher-Yates (Durstenfeld): for
// i = n-1 .. 1, swap a[i] with a[j], j = bounded(draw k, i+1), k = n-1-i.
// Sequential by definition (about 10 ns per element on a server core).
void edpp_gen_permutation_i32(int32_t *out, int64_t n, uint64_t seed) {
  parallel_for(n, [=](int64_t i) { out[i] = static_cast<int32_t>(i); });
  for (int64_t i = n - 1; i > 0; --i) {
    const int64_t j = static_cast<int64_t>(bounded(draw(seed, static_cast<uint64_t>(n - 1 - i)),
                                                   static_cast<uint64_t>(i + 1)));
    std::swap(out[i], out[j]);
  }
}

// Inputs of a batch of segments (same layout as edpp_segment: offset,
// length, op, buckets, reserved), filled in parallel over segments; segment i
// uses seeds derived from (seed, i):
//   op 0 (scan):   in0 uniform in [0,100]
//   op 1 (split):  in0 keys uniform over [0,2^31), in1 = local index
//   op 2 (gather): in0 uniform int32, in1 a Fisher-Yates permutation of
//                  [0, length)
void edpp_gen_batch_inputs(const void *segs_v, int num_segs, uint64_t seed, int32_t *in0,
                           int32_t *in1) {
  struct Seg {
    int64_t offset;
    int32_t length, op, buckets, reserved;
  };
  const Seg *segs = static_cast<const Seg *>(segs_v);
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  if (nt > 64) nt = 64;
  std::atomic<int> next{0};
  std::vector<std::thread> ts;
  for (unsigned t = 0; t < nt; ++t) {
    ts.emplace_back([&] {
      for (int i = next++; i < num_segs; i = next++) {
        const Seg &s = segs[i];
        const uint64_t sd = mix64(seed * 0x100000001B3ull + static_cast<uint64_t>(i));
        int32_t *a = in0 + s.offset;
        int32_t *b = in1 + s.offset;
        const int64_t n = s.length;
        if (s.op == 0) {
          for (int64_t k = 0; k < n; ++k) a[k] = static_cast<int32_t>(bounded(draw(sd, k), 101));
          for (int64_t k = 0; k < n; ++k) b[k] = 0;
        } else if (s.op == 1) {
          for (int64_t k = 0; k < n; ++k) a[k] = static_cast<int32_t>(draw(sd, k) >> 33);
          for (int64_t k = 0; k < n; ++k) b[k] = static_cast<int32_t>(k);
        } else {
          for (int64_t k = 0; k < n; ++k) a[k] = static_cast<int32_t>(draw(sd, k) >> 32);
          for (int64_t k = 0; k < n; ++k) b[k] = static_cast<int32_t>(k);
          const uint64_t sp = sd ^ 0x2545F4914F6CDD1Dull;
          for (int64_t k = n - 1; k > 0; --k) {
            const int64_t j = static_cast<int64_t>(
                bounded(draw(sp, static_cast<uint64_t>(n - 1 - k)), static_cast<uint64_t>(k + 1)));
            std::swap(b[k], b[j]);
          }
        }
      }
    });
  }
  for (auto &t : ts) t.join();
}

}  // extern "C"
