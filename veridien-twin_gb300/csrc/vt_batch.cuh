// Batched multi-pose rendering (vt_batch.cu): device buffers of one batch wave and the per-camera launch sequence.
#pragma once

#include "vt_wave.cuh"

namespace vtk {

struct BatchWave {
  WaveBufs shared;             // shared paths of a wave (n_pw pixels x spp)
  WaveBufs pairs;              // re-traced (path, pose) pairs, capacity cap
  uint64_t* dirty;             // per shared path: poses to re-trace
  uint32_t* off;               // per shared path: index of its first pair
  uint32_t* blk;               // per 1024 shared paths: pair count, then offset
  uint32_t* pair_src;          // per pair: shared path
  uint32_t* pair_pose;         // per pair: pose
  float4* pix;                 // per pixel of the wave: shared value
  uint64_t* pixmask;           // per pixel of the wave: OR of its sub-samples' dirty masks
  uint32_t* status;            // [0]: largest pair count of a wave (above cap: the batch must be re-run)
  unsigned long long* stats;   // [0]: pairs traced
  uint32_t n_pw, cap;
};

// read-only view of a wave's results for the per-pose finalize
struct BatchView {
  const float4* pix;
  const uint64_t* pixmask;
  const uint64_t* dirty;
  const uint32_t* off;
  const float4* shared_L;
  const float4* pair_L;
  uint32_t cap;
};

// outputs of one camera: frames [pose][h][w]
struct BatchOut {
  float4* radiance;            // or null
  uint16_t* raw;               // or null
  const uint32_t* sensor;      // device copy of the camera's sensor uniform (64 words)
  uint32_t frame0;             // pose q exposes frame frame0 + q
  float optics_scale;
  int fused;                   // raw DN computed in the finalize (no optics blur)
};

size_t batch_wave_bytes(uint32_t P, uint32_t n_pw, uint32_t cap, uint32_t n_light);
BatchWave batch_carve(void* base, uint32_t P, uint32_t n_pw, uint32_t cap, uint32_t n_light, uint32_t* counts, uint32_t* status,
                      unsigned long long* stats);
void batch_camera(const vtd::Scene& S, const CamParams& cp, const BatchCull& bc, const BatchWave& bw, uint32_t n_poses, const BatchOut& out,
                  int blocks, cudaStream_t st, uint64_t* launches);

}  // namespace vtk
