// Node-radiosity Jacobi for one right-hand side that allocates nothing (vt_radiosity_solve_static in vtwin.h).
//
// Who needs it: callers that must not allocate device memory while they run. A per-frame update loop with a fixed
// time budget cannot afford cudaMalloc/cudaFree, which may synchronise the whole device and take an unbounded time;
// a host that shares the GPU with other processes and sizes all of its device memory at start-up cannot risk an
// allocation failing in the middle of a session. Those callers own F, rho, E and B in device memory they allocated up
// front, and this entry point adds no allocation of its own: its scratch (the two Jacobi iterates and the per-block
// residual sums) is a file-scope device array of fixed size that every GPU which loads this library holds until the
// process exits.
//
// The array's name in host code is only a host-side stand-in, so the kernels get its device address from
// cudaGetSymbolAddress, looked up once per device, with that device current, on the first call made on that device.
// Every call shares the one array: calls that overlap on the GPU (two streams, or two host threads) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "vt_kernels.cuh"

namespace {

constexpr uint32_t kMaxN = VT_STATIC_SOLVE_MAX_N;
constexpr uint32_t kMaxBlocks = (kMaxN + 7) / 8;                 // jacobi_matvec: 8 rows (warps) per 256-thread block
constexpr size_t kIterBytes = size_t(kMaxN) * sizeof(float);
constexpr size_t kPartialBytes = size_t(kMaxBlocks) * 2 * sizeof(double);
constexpr size_t kScratchBytes = 2 * kIterBytes + kPartialBytes + 2 * sizeof(double);

// B0 | B1 | partial sums (2 doubles per block) | the two norms
__device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// true for memory of device `dev` (device or managed memory allocated against it): the kernels run on `dev`, and
// another GPU's memory would be an illegal address there with peer access off
bool on_device(const void* p, int dev) {
  cudaPointerAttributes a;
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == dev;
}

}  // namespace

extern "C" vt_status vt_radiosity_solve_static(const float* F, const float* rho, const float* E, float* B, uint32_t n, uint32_t max_iters,
                                               uint32_t check_every, double tol, void* stream, uint32_t* iters, double* residual) {
  if (n == 0 || n > kMaxN) return VT_ERR_ARG;                        // the static scratch holds at most kMaxN nodes
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) { cudaGetLastError(); return VT_ERR_NO_DEVICE; }
  if (!on_device(F, dev) || !on_device(rho, dev) || !on_device(E, dev) || !on_device(B, dev)) return VT_ERR_ARG;
  unsigned char* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) { cudaGetLastError(); return VT_ERR_CUDA; }
      g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float* B0 = reinterpret_cast<float*>(scratch);
  float* B1 = reinterpret_cast<float*>(scratch + kIterBytes);
  double* partials = reinterpret_cast<double*>(scratch + 2 * kIterBytes);
  double* norms = reinterpret_cast<double*>(scratch + 2 * kIterBytes + kPartialBytes);
  // the array keeps the previous call's contents: start from E and clear the sums
  if (cudaMemcpyAsync(B0, E, size_t(n) * sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess) return VT_ERR_CUDA;
  if (cudaMemsetAsync(partials, 0, kPartialBytes + 2 * sizeof(double), st) != cudaSuccess) return VT_ERR_CUDA;
  const uint32_t check = check_every ? check_every : 8;
  const uint32_t max_it = max_iters ? max_iters : 1000;
  float* cur = B0;
  float* nxt = B1;
  uint32_t it = 0, np = 0;
  double res = INFINITY;
  while (it < max_it) {
    const uint32_t k = check < max_it - it ? check : max_it - it;
    for (uint32_t j = 0; j < k; j++) {
      vtk::launch_jacobi_matvec(F, rho, E, cur, nxt, n, partials, &np, st);
      float* t = cur; cur = nxt; nxt = t;
    }
    it += k;
    vtk::launch_reduce_partials(partials, np, norms, st);
    if (cudaGetLastError() != cudaSuccess) return VT_ERR_CUDA;
    double h[2] = {0.0, 0.0};
    if (cudaMemcpyAsync(h, norms, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess) return VT_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return VT_ERR_CUDA;
    res = h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
    if (res <= tol) break;
  }
  if (cudaMemcpyAsync(B, cur, size_t(n) * sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess) return VT_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return VT_ERR_CUDA;
  if (iters) *iters = it;
  if (residual) *residual = res;
  return res <= tol ? VT_OK : VT_ERR_NOT_CONVERGED;
}
