// gbns_static.cu -- live-point counting without any device allocation.
//
// Some callers cannot call cudaMalloc: a host runtime that owns every byte of device memory
// through its own allocator (a JAX/XLA FFI custom call receives its buffers from XLA and may
// not allocate beside it), a real-time pipeline that cannot afford cudaMalloc's implicit
// device-wide synchronisation, or an embedded deployment that forbids allocation after
// start-up.  gbns_count_crossed_edges_static serves them: the caller passes only inputs and
// outputs, and the sort and out-degree scratch live in the file-scope arrays below, which
// every GPU that loads libgbns.so holds until the process exits (5 MiB per device).
#include <mutex>
#include <cstdio>
#include "gbns_device.cuh"
#include "gbns_launch.h"

// Largest sample count the static scratch holds: N + 1 node keys (two 8-byte ping-pong
// buffers) and N + 1 out-degree counters.
#define GBNS_STATIC_MAX_SAMPLES 262143

static __device__ __align__(256) unsigned long long g_static_sort[2 * (GBNS_STATIC_MAX_SAMPLES + 1)];
static __device__ __align__(256) int g_static_deg[GBNS_STATIC_MAX_SAMPLES + 1];

namespace {

int fail(int code, const char *fmt, const char *detail) {
  char msg[320];
  std::snprintf(msg, sizeof(msg), fmt, detail);
  gbns::record_error(msg);
  return code;
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
bool g_ready[kMaxDevices] = {false};
void *g_sort_ptr[kMaxDevices] = {nullptr};
void *g_deg_ptr[kMaxDevices] = {nullptr};

// Device addresses of the static scratch on the current device.  The host-side names of the
// arrays are not device addresses, so they are looked up once per device, with that device
// current.  The cache is keyed by device index only: the addresses are those of the CUDA
// runtime's primary context, and they do not survive cudaDeviceReset.
int scratch_for_current_device(void **sort, void **deg) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    return fail(-2, "gbns_count_crossed_edges_static: cudaGetDevice: %s", cudaGetErrorString(e));
  }
  if (dev < 0 || dev >= kMaxDevices) {
    return fail(-1, "gbns_count_crossed_edges_static: device index %s out of range", dev < 0 ? "<0" : ">=64");
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_ready[dev]) {
    void *p = nullptr, *q = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_sort);
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&q, g_static_deg);
    if (e != cudaSuccess) {
      return fail(-2, "gbns_count_crossed_edges_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    }
    g_sort_ptr[dev] = p;
    g_deg_ptr[dev] = q;
    g_ready[dev] = true;
  }
  *sort = g_sort_ptr[dev];
  *deg = g_deg_ptr[dev];
  return 0;
}

}  // namespace

extern "C" {

// count_crossed_edges for N <= GBNS_STATIC_MAX_SAMPLES samples with no allocation and no
// caller-provided scratch.  The first call on a device looks up the scratch address on that
// device; make that first call before any stream capture.  All calls share one scratch
// region per device and it keeps the previous call's contents: the kernel clears the
// out-degree counters itself and overwrites the sort buffers before reading them.  Calls
// whose executions overlap on the GPU (different streams, or different host threads without
// ordering) race on the shared scratch and must be serialised by the caller.
int gbns_count_crossed_edges_static(const int *sender_dev, const float *log_L_dev, long long N,
                                    int *samples_indices_dev, int *num_live_points_dev, void *stream) {
  if (N < 0 || N > GBNS_STATIC_MAX_SAMPLES)
    return fail(-1, "gbns_count_crossed_edges_static: N must be in [0, 262143] (the static scratch capacity); "
                    "use gbns_count_crossed_edges with caller-provided scratch for %s", "larger sample sets");
  if ((N > 0 && (!sender_dev || !log_L_dev)) || !samples_indices_dev || !num_live_points_dev)
    return fail(-1, "gbns_count_crossed_edges_static: %s", "NULL argument");
  void *sort = nullptr, *deg = nullptr;
  int rc = scratch_for_current_device(&sort, &deg);
  if (rc) return rc;
  cudaError_t e = gbns::launch_count_crossed_edges(sender_dev, log_L_dev, N, samples_indices_dev, num_live_points_dev,
                                                   (long long *)sort, (int *)deg, (cudaStream_t)stream);
  if (e != cudaSuccess) return fail(-2, "gbns_count_crossed_edges_static: launch: %s", cudaGetErrorString(e));
  return 0;
}

}  // extern "C"
