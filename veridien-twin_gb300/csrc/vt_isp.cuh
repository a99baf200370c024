// Buffers and launcher of the camera sensor chain (vt_isp.cu).
#pragma once

#include "vt_kernels.cuh"

namespace vtk {

struct IspBufs {
  const float4* L;   // radiance (w x h)
  const float* ri;   // relative illumination x vignetting (w x h)
  float4* A;         // the noise-reduced image (with sharpening on)
  float4* B;         // demosaiced, white-balanced, colour-corrected linear RGB
  float4* GA;        // glare level (ceil(w / F) x ceil(h / F)), two buffers
  float4* GB;
  float* raw;        // raw DN (w x h)
  uchar4* out;       // 8-bit RGB (alpha 255)
  uint8_t* yuv;      // Y (w x h), then Cb and Cr (ceil(w/2) x ceil(h/2) each)
  uint32_t* stats;   // luma sum, white-balance sums R, G, B
};

// the whole chain for one frame of the uniform's size; returns the number of kernels launched
int launch_isp(const SensorParams& P, const IspBufs& b, cudaStream_t st);

// the raster pass's display look (vt_lite_display): du as lite_nodes/renderer.js:892 writes it, the previous frame's
// statistics; stats receives this frame's (luma sum, count)
struct LiteDisplay { float du[20]; uint32_t prev[4]; uint32_t W, H; };
void launch_lite_display(const LiteDisplay& P, const float4* L, uchar4* out, uint32_t* stats, cudaStream_t st);

}  // namespace vtk
