// Kernel entry points and their launch parameters (shared by the .cu files and vt_api.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>

#include "vt_device.cuh"

namespace vtk {

// A launch size that depends only on the device (its SM count, a kernel's occupancy), computed once per device id
// into a caller's table of atomics. Host threads that race on a device's first call compute the same value, so
// the race is benign; a device id beyond the table is computed on every call.
constexpr int MAX_DEVICES = 64;
template <class Fn>
inline int per_device_value(std::atomic<int> (&table)[MAX_DEVICES], Fn compute) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); dev = 0; }
  if (dev < 0 || dev >= MAX_DEVICES) return std::max(1, compute(dev));
  int v = table[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    v = std::max(1, compute(dev));
    table[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}
inline int device_sms(int dev) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) { cudaGetLastError(); sms = 1; }
  return std::max(1, sms);
}

// one camera dispatch (the fields of gpu/renderer.js:888 _packCam that the estimators read)
struct CamParams {
  float rx[3], ry[3], rz[3], pos[3];   // camera axes in the dome frame (columns of R_D_C) and centre
  vtd::Kb4 lens;
  uint32_t w, h, spp, seed, cam_index, options, skip, n_light, mode, max_depth, root;
  float t0, t1, scale;
  uint32_t tile_w, tile_h;             // pixel enumeration order: tiles of tile_w x tile_h (product 32)
  uint32_t refill;                     // traversal lanes: a warp takes new rays once this many of its lanes are idle
  uint32_t refine;                     // pass-2 extra sub-samples (camRefine), 0 none
};

// default pixel tile: consecutive paths are neighbouring pixels of an 8 x 4 tile
constexpr int TILE_W = 8, TILE_H = 4;
// default refill threshold of the persistent traversal lanes
constexpr uint32_t REFILL = 8;
// padded pixel count of a w x h image in tile_w x tile_h tiles
inline uint32_t tiled_pixels(uint32_t w, uint32_t h, uint32_t tw, uint32_t th) { return ((w + tw - 1) / tw) * ((h + th - 1) / th) * tw * th; }
void launch_trace(const vtd::Scene& S, const float4* o4, const float4* d4, uint32_t n, uint32_t mask, uint32_t any_hit, uint32_t root,
                  float4* out4, float* out_v, cudaStream_t st);
void launch_visible(const vtd::Scene& S, float3 c, const float3* pts, uint32_t n, float tol, float time, uint32_t skip, uint8_t* out,
                    cudaStream_t st);

// sensor (gpu/wgsl/sensor.wgsl.js:177 sensorExpose)
struct SensorParams { uint32_t w[64]; };
void launch_sensor_expose(const SensorParams& su, const float4* E, float scale, float* raw, cudaStream_t st);
// the same with raw DN stored as uint16 (ADC depth <= 16 bits)
void launch_sensor_expose_u16(const SensorParams& su, const float4* E, float scale, uint16_t* raw, cudaStream_t st);

// radiosity
// B_out = E + rho (F B_in), n x 1, and per-block partial sums of |B_out - B_in|^2 and |B_out|^2 (doubles)
void launch_jacobi_matvec(const float* F, const float* rho, const float* E, const float* Bin, float* Bout, uint32_t n,
                          double* partials, uint32_t* n_partials, cudaStream_t st);
// the same with F's rows fed into shared memory by bulk copies (n % 4 == 0); bounded waits raise matvec_error
void launch_jacobi_matvec_tma(const float* F, const float* rho, const float* E, const float* Bin, float* Bout, uint32_t n,
                              double* partials, uint32_t* n_partials, cudaStream_t st);
uint32_t jacobi_matvec_tma_blocks(uint32_t n);
// nonzero when a bulk copy of the TMA-fed matvec did not land in time (and reset it)
uint32_t matvec_error(cudaStream_t st, bool reset);
// B_out = E + rho (F B_in), n x R row-major (R <= 64, multiple of 4), CUDA-core FP32 GEMM
// work: jacobi_gemm_fp32_work(n, R) bytes for the split-K partial products (null: no split)
size_t jacobi_gemm_fp32_work(uint32_t n, uint32_t R);
void launch_jacobi_gemm_fp32(const float* F, const float* rho, const float* E, const float* Bin, float* Bout, uint32_t n, uint32_t R,
                             float* work, double* partials, uint32_t* n_partials, cudaStream_t st);
// sum the partials into out[0..1] (deterministic order)
void launch_reduce_partials(const double* partials, uint32_t n, double* out, cudaStream_t st);
void launch_form_factors(uint32_t n, const float* C, const float* N, const float* A, float* F, cudaStream_t st);
// the same with each pair's visibility through the scene: K rays per unordered pair (K <= 255, n <= 65535);
// counts: n x n bytes of work, head: one word
void launch_form_factors_visible(const vtd::Scene& S, uint32_t n, const float* C, const float* N, const float* A, uint32_t K, uint32_t* head,
                                 uint8_t* counts, float* F, int blocks, cudaStream_t st);

}  // namespace vtk
