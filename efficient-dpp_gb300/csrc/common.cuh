// common.cuh — shared device helpers for the sm_103a primitives:
// status plumbing, the device fault word, bounded waits on %globaltimer,
// and inline-PTX wrappers for mbarriers and 1-D TMA bulk copies
// (cp.async.bulk) between global and shared memory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "edpp.h"

namespace edpp {

// Lanes of the calling warp whose value has the same low `bits` bits as this
// lane's, restricted to `among`; one vote per bit (all 32 lanes must call).
// Used instead of __match_any_sync, which on this GPU issues far slower.
__device__ __forceinline__ unsigned match_low_bits(unsigned v, int bits, unsigned among) {
  unsigned peers = among;
  for (int i = 0; i < bits; ++i) {
    const unsigned one = (v >> i) & 1u;
    const unsigned bb = __ballot_sync(0xffffffffu, one);
    peers &= one ? bb : ~bb;
  }
  return peers;
}


// Number of SMs on a GB300 (two dies of 76).  Grids are sized as multiples of
// the SM count the runtime reports; this is only the fallback.
constexpr int kGb300Sms = 152;

// Default limit of any device-side wait, in nanoseconds.
constexpr uint64_t kDefaultWaitNs = 2000000000ull;  // 2 s

// The device fault word lives in status.cu (one per device); kernels get its
// address as an argument (host side: fault_word()).
__device__ __forceinline__ void raise_fault(unsigned *fault, unsigned bits) {
  atomicOr(fault, bits);
}

__device__ __forceinline__ bool fault_raised(const unsigned *fault) {
  return *(const volatile unsigned *)fault != 0u;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---- memory-model helpers -------------------------------------------------

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(uint64_t *p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_acquire_u64(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(uint64_t *p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// ---- mbarrier + TMA bulk copy (1-D, non-tensor) ----------------------------

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Make mbarrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this thread's generic-proxy shared-memory writes before later
// async-proxy (TMA) accesses of the same bytes.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for phase `parity` of `bar` to complete; gives up after timeout_ns,
// raising EDPP_FAULT_TMA.  Returns false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint64_t timeout_ns, unsigned *fault) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (globaltimer_ns() - t0 > timeout_ns) {
      raise_fault(fault, EDPP_FAULT_TMA);
      return false;
    }
  }
  return true;
}

// Bulk copy global -> shared, completion signalled on `bar` (tx bytes).
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void tma_load_1d(void *smem_dst, const void *gmem_src, uint32_t bytes,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Same, with an L2 evict-first hint for data read once.
__device__ __forceinline__ void tma_load_1d_evict_first(void *smem_dst, const void *gmem_src,
                                                        uint32_t bytes, uint64_t *bar,
                                                        uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], "
      "%2, [%3], %4;" ::"r"(smem_addr(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_addr(bar)), "l"(policy)
      : "memory");
}

__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// 16-byte global load with an L2 eviction-priority policy (createpolicy).
__device__ __forceinline__ uint4 ld_v4_policy(const uint4 *p, uint64_t policy) {
  uint4 v;
  asm volatile("ld.global.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p), "l"(policy));
  return v;
}

// Bulk copy shared -> global (bulk-group completion).
__device__ __forceinline__ void tma_store_1d(void *gmem_dst, const void *smem_src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gmem_dst),
               "r"(smem_addr(smem_src)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_store_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// Wait until all committed bulk stores have finished reading shared memory.
__device__ __forceinline__ void tma_store_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// Wait until all committed bulk stores are complete (visible in global).
__device__ __forceinline__ void tma_store_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// ---- host helpers ----------------------------------------------------------

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

inline int cuda_status(cudaError_t e) { return e == cudaSuccess ? EDPP_OK : EDPP_ECUDA; }

// Launch-error check after a kernel launch.
inline int launch_status() { return cuda_status(cudaGetLastError()); }

// SM count of the current device (cached per device).
int device_sm_count();

// L2 size of the current device in bytes (cached).
int device_l2_bytes();

// Device address of the fault word of the current device (cached).
unsigned *fault_word();

__host__ __device__ __forceinline__ int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ __forceinline__ int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }

// Round x up to a multiple of a.
__host__ __device__ constexpr inline size_t round_up(size_t x, size_t a) {
  return (x + a - 1) / a * a;
}

}  // namespace edpp
