// Differentiable calibration render (vt_calib.cu): the forward estimator, its path-replay adjoint, and the node
// radiosity pieces of the calibration model (direct transfer from the emitter triangles, transposed Jacobi).
#pragma once

#include "vt_wave.cuh"

namespace vtk {

constexpr uint32_t CAL_MAX_DEPTH = 4, CAL_MAX_NL = 4;

// parameters, node data and accumulators of one calibration render (device pointers)
struct CalibDev {
  const float* albedo;          // n_mat x 3
  const float* lamp;            // n_lamps: radiance of each emitter triangle
  const uint32_t* emit_of_tri;  // per triangle slot: emitter index, or ~0
  const uint32_t* tri_node;     // per static triangle slot: node
  const float* H;               // 3 x n_nodes (planar): irradiance at the node from the other nodes' radiosity (F B)
  uint32_t n_static_tris, n_mat, n_lamps, n_nodes;
  const float4* target;         // this camera's target image, w x h row-major
  float4* image;                // this camera's image: written by the forward, read by the backward
  double inv_count;             // 1 / (3 x pixels of all cameras in the loss)
  double* partials;             // forward: per-block loss sums
  double* g_albedo;             // backward accumulators (FP64)
  double* g_lamp;
  double* g_H;                  // 3 x n_nodes
  double* g_K;                  // this camera's 8 intrinsics (fx, fy, cx, cy, k1..k4): the image loss's derivative
};

// stored-path form: the wavefront forward of one camera (records of all its paths kept, path (i, id) at
// records[i n_pix + id]), the image and per-block loss partials (returns their number); and the backward from the
// records, without tracing
size_t calib_record_bytes(uint32_t paths);
// with `tangents` (calib_tan_bytes per path, NULL: none) the forward also keeps each path's derivative record in its
// primary direction, and the backward then adds the derivative in the camera's intrinsics (C.g_K)
size_t calib_tan_bytes(uint32_t paths);
uint32_t calib_wave_forward(const vtd::Scene& S, const CamParams& cp, const CalibDev& C, WaveBufs wb, uint32_t wave_paths, void* records,
                            void* tangents, int blocks, cudaStream_t st);
void calib_records_backward(const CamParams& cp, const CalibDev& C, const void* records, const void* tangents, int blocks, cudaStream_t st);
// the recorded paths' discrete decisions (for checking): per path in (row, column, sub-sample) order, CAL_MAX_DEPTH x
// (triangle, instance) and CAL_MAX_DEPTH x CAL_MAX_NL light-sample weights q (0: occluded or no contribution)
void calib_export_paths(const CamParams& cp, const void* records, const void* tangents, uint32_t* tri_inst, float* q, cudaStream_t st);
// replay form: the paths of the camera's sub-samples [i0, i1) traced into `records` (and `tangents`, NULL: none) at
// records[(i - i0) n_pix + id], then mode 0 adds their values to the image (the chunk ending at spp writes the image
// and the per-block loss partials, whose number it returns), 1 accumulates the gradients of the image loss
// (albedos, emitter radiances, node light), 2 also the derivative in the camera's intrinsics (C.g_K). The image of
// the forward's chunks is the stored form's image bit for bit.
//
// `decisions` (calib_dec_bytes per path of the camera, at decisions[i n_pix + id]; NULL: none) keeps each path's
// discrete decisions: per bounce the triangle and instance the extension ray met, per vertex and light sample
// whether the shadow ray was occluded. dec_mode 1 records them while tracing; dec_mode 2 replays them: the extension
// rays meet the recorded triangles (one intersection each, the traversal's own arithmetic) and the occluded samples
// are cleared without shadow rays, so the records are the traced ones bit for bit.
uint32_t calib_wave_chunk(const vtd::Scene& S, const CamParams& cp, const CalibDev& C, WaveBufs wb, uint32_t wave_paths, void* records,
                          void* tangents, uint32_t i0, uint32_t i1, int mode, int blocks, cudaStream_t st, void* decisions = nullptr,
                          int dec_mode = 0);
size_t calib_dec_bytes(uint32_t paths);
// D[i][t]: irradiance at node i (centre, normal) from emitter triangle t at unit radiance, with visibility
void launch_direct_transfer(const vtd::Scene& S, const float* centres, const float* normals, uint32_t n, uint32_t n_lamps,
                            uint32_t samples, float* D, cudaStream_t st);
// y = D L (n x n_lamps times n_lamps)
void launch_dl(const float* D, const float* L, uint32_t n, uint32_t n_lamps, float* y, cudaStream_t st);
// one transposed Jacobi sweep of the adjoint: lam_out = F^T (g + rho o lam_in), FP64 vectors; work: splits x n doubles
void launch_jacobi_t(const float* F, const double* g, const float* rho, const double* lam_in, double* lam_out, uint32_t n, double* work,
                     cudaStream_t st);
size_t jacobi_t_work(uint32_t n);
// y = a o b (n floats)
void launch_mul(const float* a, const float* b, float* y, uint32_t n, cudaStream_t st);
// the calibration model's node radiosity for the three channels at once: B_c = rho_c o (DL + F B_c) by `iters`
// Jacobi sweeps from B_c = rho_c o DL, at FP64 accuracy (F in FP32; float-pair products and sums), then H_c = F B_c
// rounded to FP32; rho and H planar 3 x n; work: at least 48 n bytes, 16-byte aligned
void launch_radiosity64(const float* F, const float* rho, const float* DL, uint32_t n, uint32_t iters, void* work, float* H, cudaStream_t st);
// sum of n doubles (deterministic order) into out
void launch_sum(const double* p, uint32_t n, double* out, cudaStream_t st);

}  // namespace vtk
