// primitives.cpp — the reference's synchronous, time-returning primitive
// API (include/edpp_primitives.hpp) on top of the C ABI (include/edpp.h).
#include "edpp_primitives.hpp"

#include <cuda_runtime.h>

#include "edpp.h"

namespace edpp {
namespace primitives {
namespace {

// Times `f` (which enqueues on the default stream) with CUDA events and
// waits for it; returns elapsed ms, or -1 on any error.
template <typename F> double timed(F f) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess) return -1;
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(a);
    return -1;
  }
  double ms = -1;
  if (cudaEventRecord(a, 0) == cudaSuccess && f() == EDPP_OK &&
      cudaEventRecord(b, 0) == cudaSuccess && edpp_sync_status(nullptr, 1) == EDPP_OK) {
    float t = 0;
    if (cudaEventElapsedTime(&t, a, b) == cudaSuccess) ms = t;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

// Stream-ordered temporary from the default pool, freed after use.
struct Temp {
  void *p = nullptr;
  size_t bytes = 0;
  explicit Temp(size_t n) : bytes(n) {
    if (n && cudaMallocAsync(&p, n, 0) != cudaSuccess) p = nullptr;
  }
  ~Temp() {
    if (p) cudaFreeAsync(p, 0);
  }
  bool ok() const { return bytes == 0 || p != nullptr; }
};

double scan_excl(const int *in, int *out, int64_t n, int algo) {
  Temp ws(edpp_scan_workspace_size(n, EDPP_I32, algo));
  if (!ws.ok()) return -1;
  return timed([&] {
    return edpp_scan_exclusive_i32(in, out, n, algo, ws.p, ws.bytes, nullptr);
  });
}

double split_any(const int *d_in, int *d_out, int *d_start, int length, int buckets,
                 DataStruc s, const int *vin, int *vout) {
  if (length < 0 || buckets < 1 || (buckets & (buckets - 1))) return -1;
  // SOA needs both value arrays (splitImpl.cpp:29-34).
  if (s == KVS_SOA && (!vin || !vout)) return -1;
  const int layout = s == KO ? EDPP_KO : (s == KVS_AOS ? EDPP_KVS_AOS : EDPP_KVS_SOA);
  Temp ws(edpp_split_workspace_size(length, buckets, layout));
  if (!ws.ok()) return -1;
  return timed([&] {
    return edpp_split_i32(d_in, d_out, d_start, length, buckets, layout, vin, vout, ws.p, ws.bytes,
                          nullptr);
  });
}

}  // namespace

// Multi-pass gather / scatter through the shared-memory-window form: the same
// results as the reference's pass-by-pass sweeps for every pass count.
double gather(const int *d_in, int *d_out, int length, const int *d_loc, int, int, int pass) {
  if (pass < 1) return -1;
  if (edpp_gather_prefers_direct(length))  // the source stays in L2: one direct sweep
    return timed([&] { return edpp_gather_i32(d_in, d_out, length, d_loc, 1, nullptr); });
  Temp ws(edpp_gather_tiled_workspace_size(length));
  if (!ws.ok()) return -1;
  return timed([&] {
    return edpp_gather_i32_tiled(d_in, d_out, length, d_loc, pass, ws.p, ws.bytes, nullptr);
  });
}

double scatter(const int *d_in, int *d_out, int length, const int *d_loc, int, int, int pass) {
  if (pass < 1) return -1;
  Temp ws(edpp_scatter_tiled_workspace_size(length));
  if (!ws.ok()) return -1;
  return timed([&] {
    return edpp_scatter_i32_tiled(d_in, d_out, length, d_loc, pass, ws.p, ws.bytes, nullptr);
  });
}

double scan_chained(const int *d_in, int *d_out, int length, int, int, int R, int L) {
  if (R == 0 && L == 0) return 1;  // scanImpl.cpp:19-22
  return scan_excl(d_in, d_out, length, EDPP_SCAN_LOOKBACK);
}

double scan_RSS(const int *d_in, int *d_out, unsigned length, int, int) {
  return scan_excl(d_in, d_out, length, EDPP_SCAN_RTS);
}

double scan_RSS_single(const int *d_in, int *d_out, unsigned length) {
  return scan_excl(d_in, d_out, length, EDPP_SCAN_RTS);
}

double scan_SSA(const int *d_in, int *d_out, uint64_t len) {
  return scan_excl(d_in, d_out, static_cast<int64_t>(len), EDPP_SCAN_SSA);
}

double scan_RTS(const int *d_in, int *d_out, uint64_t len) {
  return scan_excl(d_in, d_out, static_cast<int64_t>(len), EDPP_SCAN_RTS);
}

double WI_split(const int *d_in, int *d_out, int *d_start, int length, int buckets,
                DataStruc structure, const int *d_in_values, int *d_out_values, int, int) {
  return split_any(d_in, d_out, d_start, length, buckets, structure, d_in_values, d_out_values);
}

double WG_split(const int *d_in, int *d_out, int *d_start, int length, int buckets, ReorderType,
                DataStruc structure, const int *d_in_values, int *d_out_values, int, int) {
  return split_any(d_in, d_out, d_start, length, buckets, structure, d_in_values, d_out_values);
}

double single_split(const int *d_in, int *d_out, int length, int buckets, bool,
                    DataStruc structure) {
  if (structure == KVS_SOA) return -1;  // splitImpl.cpp:376-379: SOA not supported
  return split_any(d_in, d_out, nullptr, length, buckets, structure, nullptr, nullptr);
}

}  // namespace primitives
}  // namespace edpp
