// nmg_static.cu -- nmg_max_dm_static: the max |m_i - m_prev_i| reduction of
// nmg_max_dm for callers that must not allocate device memory.
//
// Who needs it: a host program whose GPU memory is owned entirely by its own
// pool (for example a framework's caching allocator that has to account for
// every byte, so a library may not cudaMalloc behind its back), or a tight
// control loop that polls convergence between integration steps and cannot
// afford cudaMalloc/cudaFree, which synchronise the whole device.  Such a
// caller already holds m and m_prev on the device and passes them in.
//
// The only scratch this needs -- one partial maximum per block -- lives in a
// file-scope __device__ array of kStaticPartials doubles (8 KB), which every
// GPU that loads the library keeps until the process exits.  Host code cannot
// use the array's name as a device address, so the first call on each device
// looks the address up with cudaGetSymbolAddress (with that device current)
// and caches it; make that first call before any stream capture.  All calls
// share the array: calls that overlap on the GPU (from several host threads
// or streams) race on it and must be serialised by the caller.  Every call
// overwrites each partial it reads, so nothing has to be cleared.  The kernel
// and the read-back run on the legacy default stream, which is not ordered
// with non-blocking streams (a handle's own stream is one): the caller makes
// sure that whatever wrote m and m_prev has finished before the call.
#include <mutex>

#include "nmg_internal.h"

namespace {

constexpr int kStaticThreads = 256;
constexpr int kNodesPerThread = 8;
constexpr int kStaticPartials = 1024;
// largest node count whose partials fit the static array
constexpr long long kStaticMaxNodes = (long long)kStaticPartials * kStaticThreads * kNodesPerThread;
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_maxdm_partials[kStaticPartials];

std::mutex g_setup_mutex;
double *g_partials_addr[kMaxDevices] = {nullptr};

// Each block covers kStaticThreads * kNodesPerThread consecutive nodes and
// writes one partial maximum (same per-node arithmetic as nmg_max_dm).
__global__ void __launch_bounds__(kStaticThreads)
    k_maxdm_static(int n, const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ part) {
  __shared__ double smem[kStaticThreads / 32];
  const long long first = (long long)blockIdx.x * kStaticThreads * kNodesPerThread;
  double mx = 0.0;
  for (int k = 0; k < kNodesPerThread; ++k) {
    const long long i = first + (long long)k * kStaticThreads + threadIdx.x;
    if (i < n) {
      const double d0 = a[3 * i] - b[3 * i], d1 = a[3 * i + 1] - b[3 * i + 1], d2 = a[3 * i + 2] - b[3 * i + 2];
      mx = fmax(mx, sqrt(d0 * d0 + d1 * d1 + d2 * d2));
    }
  }
  for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) smem[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < kStaticThreads / 32; ++w) r = fmax(r, smem[w]);
    part[blockIdx.x] = r;
  }
}

int static_fail(int code, const std::string &msg) {
  nmg::set_handleless_error(msg);  // read back with nmg_last_error(NULL)
  return code;
}

}  // namespace

extern "C" int nmg_max_dm_static(const double *d_m, const double *d_m_prev, int n_nodes, double *out) {
  if (!d_m || !d_m_prev || !out) return static_fail(-1, "nmg_max_dm_static: NULL pointer");
  if (n_nodes <= 0) return static_fail(-2, "nmg_max_dm_static: n_nodes must be positive");
  if (n_nodes > kStaticMaxNodes)
    return static_fail(-2, "nmg_max_dm_static: n_nodes " + std::to_string(n_nodes) + " exceeds the static scratch "
                               "limit of " + std::to_string(kStaticMaxNodes) + " nodes");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return static_fail(101, "nmg_max_dm_static: no usable CUDA device");
  double *part = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_addr[dev]) {
      // one-time set-up on this device (the device is current here)
      cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void **>(&g_partials_addr[dev]), g_maxdm_partials);
      if (e != cudaSuccess) {
        g_partials_addr[dev] = nullptr;
        return static_fail(100, std::string("nmg_max_dm_static: cudaGetSymbolAddress failed: ") +
                                    cudaGetErrorString(e));
      }
    }
    part = g_partials_addr[dev];
  }
  const long long per_block = (long long)kStaticThreads * kNodesPerThread;
  const int blocks = (int)((n_nodes + per_block - 1) / per_block);
  k_maxdm_static<<<blocks, kStaticThreads>>>(n_nodes, d_m, d_m_prev, part);
  // a launch that did not start leaves the previous call's partials in the
  // array: report it instead of returning their stale maximum
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return static_fail(100, std::string("nmg_max_dm_static: launch failed: ") + cudaGetErrorString(e));
  double host[kStaticPartials];
  e = cudaMemcpy(host, part, sizeof(double) * blocks, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess)
    return static_fail(100, std::string("nmg_max_dm_static: ") + cudaGetErrorString(e));
  double mx = 0.0;
  for (int b = 0; b < blocks; ++b) mx = host[b] > mx ? host[b] : mx;
  *out = mx;
  return 0;
}
