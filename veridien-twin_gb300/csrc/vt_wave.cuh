// Wavefront path-state buffers and launchers (vt_wave.cu).
#pragma once

#include "vt_kernels.cuh"

namespace vtk {

// structure-of-arrays path state of one wave, carved from one device allocation
struct WaveBufs {
  float4* o;        // ray origin, time
  float4* d;        // ray direction, pdf of the BSDF sample that made it
  float4* thr;      // path throughput
  float4* L;        // radiance of the sub-sample so far, key bits (w)
  float4* hit;      // t, u, v, triangle bits
  float4* nee;      // throughput at the vertex whose light samples are pending, time
  uint4* meta;      // pixel id, sub-sample index, pixel hash, bounce (0: no pixel)
  uint32_t* hinst;  // instance of the hit
  uint32_t* qa;     // ray queues (path ids), alternating per bounce
  uint32_t* qb;
  uint32_t* q_sh;   // paths with light samples to test
  float4* sh;       // per path and light sample: (shadow origin, tmax) (direction, valid) (contribution)
  float4* acc;      // per pixel running sum across waves, key bits
  uint32_t* counts; // queue lengths
  // the current bounce's view
  uint32_t* q_in;
  uint32_t* q_out;
  uint32_t* count_in;
  uint32_t* count_out;
  uint32_t* count_sh;
};

size_t wave_bytes(uint32_t paths, uint32_t n_light, uint32_t n_pix);
WaveBufs wave_carve(void* base, uint32_t paths, uint32_t n_light, uint32_t n_pix, uint32_t* counts);
void wave_render(const vtd::Scene& S, const CamParams& cp, WaveBufs wb, uint32_t wave_paths, float4* out, int blocks, cudaStream_t st,
                 uint64_t* launches);
int wave_blocks_per_sm();

}  // namespace vtk
