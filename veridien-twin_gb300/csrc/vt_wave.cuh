// Wavefront path-state buffers and launchers (vt_wave.cu), and the pose-batch extensions (vt_batch.cu).
#pragma once

#include "vt_kernels.cuh"

namespace vtk {

// Kernel variants of the wavefront:
//   WAVE_PLAIN   one pose: every path traced against the whole scene
//   WAVE_SHARED  a pose batch's shared paths: bodies whose pose varies across the batch are skipped, and every
//                segment is tested against all poses' copies of them (BatchCull) to mark the poses whose result
//                may differ from the shared one
//   WAVE_PAIRS   the (path, pose) pairs so marked, each traced whole against its own pose's scene uniform
enum { WAVE_PLAIN = 0, WAVE_SHARED = 1, WAVE_PAIRS = 2 };

// pose-batch data of the wavefront kernels
struct BatchCull {
  const float4* nodes;      // BVH over (pose, body) items: 2 float4 per node (lo, first|left bits) (hi, count bits; 0 = interior)
  const float4* items;      // 4 float4 per item: (box lo, pose bits) (box hi, body bits) (capsule a, r) (capsule b, -)
  uint32_t n_nodes;
  uint32_t vary;            // bodies whose pose differs across the batch
  const float* su_base;     // per-pose scene uniforms (WAVE_PAIRS)
  uint32_t su_stride;       // words per uniform
  uint64_t* dirty;          // per shared path: poses whose result may differ (WAVE_SHARED)
  const uint32_t* pair_pose;// per pair path: its pose (WAVE_PAIRS)
  const uint32_t* pair_src; // per pair path: the shared path it repeats (WAVE_PAIRS)
  uint32_t n_pw;            // pixels of the batch wave (pixel id = px0 + path % n_pw, sub-sample = path / n_pw)
  uint32_t px0;
};

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
  float4* acc2;     // per refined pixel: running sum of the refinement waves
  uint32_t* rlist;  // refined pixel ids
  uint32_t* rcount; // their number (refinement only)
  uint32_t* counts; // queue lengths
  // the current bounce's view
  uint32_t* q_in;
  uint32_t* q_out;
  uint32_t* count_in;
  uint32_t* count_out;
  uint32_t* count_sh;
  uint32_t* fetch;  // next queue entry to take, for the persistent traversal kernels (zeroed before each)
  // static first-hit cache of a fixed camera (null: off): per (sub-sample i, pixel id) at i * hc_stride + id the
  // closest hit in the static BVH (t, u, v, triangle bits), t = 0 while empty
  float4* hcache;
  uint32_t hc_stride, hc_cap;   // pixel ids per sub-sample, sub-samples held
  // static-occlusion cache of a fixed camera with a still emitter (null: off), indexed like hcache: per first-hit
  // light sample j bit j set when the static scene hides it, bit 31 once the word is valid
  uint32_t* scache;
  unsigned long long* stats;   // optional: [0] rays of the closest-hit kernels, [1] paths of the any-hit kernels
  BatchCull bc;
};

// optional events around the bounce kernels (kernel profiling): pairs in launch order, kind 0 extend, 1 shade, 2 shadow
struct KernelTimer {
  cudaEvent_t* ev;
  uint8_t* kind;
  int cap, n;
};

size_t wave_bytes(uint32_t paths, uint32_t n_light, uint32_t n_pix);
WaveBufs wave_carve(void* base, uint32_t paths, uint32_t n_light, uint32_t n_pix, uint32_t* counts);
// one camera: pass 1 (cp.spp sub-samples per pixel), then when cp.refine > 0 pass 2 over the selected pixels with
// cp2 (the refinement's light samples) continuing the sub-sample sequences
void wave_render(const vtd::Scene& S, const CamParams& cp, WaveBufs wb, uint32_t wave_paths, float4* out, int blocks, cudaStream_t st,
                 uint64_t* launches, KernelTimer* timer = nullptr, const CamParams* cp2 = nullptr);
int wave_blocks_per_sm();

// one wave's bounces (extend, shade, shadow per bounce) over the paths queued in wb.qa / counts[0]
void wave_bounces(const vtd::Scene& S, const CamParams& cp, WaveBufs wb, int var, int blocks, cudaStream_t st, uint64_t* launches,
                  KernelTimer* timer = nullptr);
// the closest-hit kernel over wb.qa / counts (plain scene) and the camera rays of sub-samples [i0, i0 + n_i) of all
// n_pix pixel ids (path p = (i - i0) n_pix + id), queued in wb.qa / counts[0]
void launch_wave_extend(const vtd::Scene& S, const CamParams& cp, const WaveBufs& wb, int blocks, cudaStream_t st);
void launch_wave_gen(const CamParams& cp, WaveBufs wb, uint32_t i0, uint32_t n_i, uint32_t n_pix, int blocks, cudaStream_t st);
// camera rays of a batch wave: paths p = i * n_pw + lp, i < spp, pixel id px0 + lp; clears the dirty masks
void wave_gen_batch(const CamParams& cp, WaveBufs wb, int blocks, cudaStream_t st);
// camera rays of the pair paths (pair j repeats shared path pair_src[j]); count in counts[0]
void wave_gen_pairs(const CamParams& cp, WaveBufs wb, int blocks, cudaStream_t st);

}  // namespace vtk
