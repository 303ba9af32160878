// status.cu — library-wide state: the device fault word, status strings,
// device queries, and the synchronous status check.
#include <mutex>

#include "common.cuh"

namespace edpp {

// One fault word per device.  Kernels receive its address (fault_word()).
__device__ unsigned int g_fault_word = 0u;

namespace {
constexpr int kMaxDevices = 64;
std::once_flag g_dev_once[kMaxDevices];
int g_sm_count[kMaxDevices];
int g_l2_bytes[kMaxDevices];
unsigned *g_fault_ptr[kMaxDevices];

int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) return 0;
  return d;
}

void init_device(int d) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || sms <= 0)
    sms = kGb300Sms;
  g_sm_count[d] = sms;
  int l2 = 0;
  if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, d) != cudaSuccess || l2 <= 0)
    l2 = 126 << 20;
  g_l2_bytes[d] = l2;
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_fault_word) != cudaSuccess) p = nullptr;
  g_fault_ptr[d] = static_cast<unsigned *>(p);
}
}  // namespace

int device_sm_count() {
  const int d = current_device();
  std::call_once(g_dev_once[d], init_device, d);
  return g_sm_count[d];
}

int device_l2_bytes() {
  const int d = current_device();
  std::call_once(g_dev_once[d], init_device, d);
  return g_l2_bytes[d];
}

unsigned *fault_word() {
  const int d = current_device();
  std::call_once(g_dev_once[d], init_device, d);
  return g_fault_ptr[d];
}

}  // namespace edpp

extern "C" {

const char *edpp_status_string(int status) {
  switch (status) {
    case EDPP_OK: return "ok";
    case EDPP_EINVAL: return "invalid argument";
    case EDPP_ENOMEM: return "workspace too small or out of memory";
    case EDPP_ETIMEOUT: return "bounded device wait expired";
    case EDPP_ECUDA: return "CUDA runtime error";
    default: return "unknown status";
  }
}

int edpp_version(void) { return 10000; /* 1.0.0 */ }

int edpp_device_fault(unsigned int *fault_bits, int clear) {
  unsigned v = 0;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return EDPP_ECUDA;
  e = cudaMemcpyFromSymbol(&v, edpp::g_fault_word, sizeof(v));
  if (e != cudaSuccess) return EDPP_ECUDA;
  if (clear) {
    const unsigned zero = 0;
    e = cudaMemcpyToSymbol(edpp::g_fault_word, &zero, sizeof(zero));
    if (e != cudaSuccess) return EDPP_ECUDA;
  }
  if (fault_bits) *fault_bits = v;
  return EDPP_OK;
}

int edpp_sync_status(void *stream, int clear) {
  cudaError_t e = cudaStreamSynchronize(edpp::as_stream(stream));
  if (e != cudaSuccess) return EDPP_ECUDA;
  e = cudaGetLastError();
  if (e != cudaSuccess) return EDPP_ECUDA;
  unsigned v = 0;
  e = cudaMemcpyFromSymbol(&v, edpp::g_fault_word, sizeof(v));
  if (e != cudaSuccess) return EDPP_ECUDA;
  if (clear && v) {
    const unsigned zero = 0;
    e = cudaMemcpyToSymbol(edpp::g_fault_word, &zero, sizeof(zero));
    if (e != cudaSuccess) return EDPP_ECUDA;
  }
  if (v & EDPP_FAULT_PLAN) return EDPP_EINVAL;
  return v ? EDPP_ETIMEOUT : EDPP_OK;
}

}  // extern "C"
