// Batched rendering of many kinematic poses of one scene (the twin's renderFrame over a pose sweep with setPoses
// per pose, gpu/renderer.js:620,986), GB300-first.
//
// Poses move a few small bodies; every other part of the scene is common to the batch. A wave of camera paths is
// traced once against the common scene (WAVE_SHARED: the varying bodies skipped) while each segment is tested
// against every pose's copy of the varying bodies with the culls trace_scene applies before it traverses a body.
// A path whose segments reach none of pose q's copies has, under pose q, exactly the result of the shared path:
// the same hits, the same light-sample visibility, the same radiance, bit for bit. The (path, pose) pairs a
// segment may reach are re-traced whole against their own pose's scene uniform (WAVE_PAIRS), and each pose's
// pixel sums take the shared or the re-traced radiance of every sub-sample, in sub-sample order. The result of the
// batch is therefore identical to rendering each pose on its own; the work is one traversal of the shared paths
// plus the pairs (a small fraction at 6 mm instruments).
//
// A batch wave is a band of whole pixels x all their sub-samples (path p = i * n_pw + lp), so one wave holds every
// term of its pixels' sums. Per wave:
//   gen -> bounces (shared) -> finalize_shared (pixel sums, OR of dirty masks) -> scan of popc(dirty)
//   -> expand (pair list ordered by path, then pose) -> gen_pairs -> bounces (pairs) -> finalize_poses
//   (per pose and pixel: radiance, and the sensor fused in when the optics blur is off)
// Every count lives on the device, so the whole sequence can be captured once in a CUDA graph and replayed.
#include <algorithm>

#include "vt_batch.cuh"
#include "vt_camera.cuh"
#include "vt_sensor.cuh"

namespace vtk {
using namespace vtd;

namespace {
constexpr int T = 256;
constexpr int SCAN = 1024;   // paths per scan block

// in-order sum of a pixel's sub-samples and its key, as wave_finalize computes it over a whole frame
struct PixSum {
  float3 s = make_float3(0.0f, 0.0f, 0.0f);
  uint32_t key = 0;
  __device__ __forceinline__ void add(uint32_t i, float4 L) {
    s = s + xyz(L);
    const uint32_t gk = __float_as_uint(L.w);
    if (i == 0) key = gk;
    else if ((gk & 0xffffu) != (key & 0xffffu)) key |= 0x40000u;
    key |= gk & 0x30000u;
  }
  __device__ __forceinline__ float4 value(const CamParams& cp) const {
    const float sc = cp.scale / float(cp.spp);
    return make_float4(s.x * sc, s.y * sc, s.z * sc, key == 0xfffeu ? 0.0f : 1.0f);
  }
};

__global__ void __launch_bounds__(T) finalize_shared_kernel(const CamParams cp, const float4* __restrict__ L, const uint64_t* __restrict__ dirty,
                                                           uint32_t px0, uint32_t n_pw, float4* __restrict__ pix, uint64_t* __restrict__ pixmask) {
  for (uint32_t lp = blockIdx.x * blockDim.x + threadIdx.x; lp < n_pw; lp += gridDim.x * blockDim.x) {
    uint32_t x, y;
    if (!pixel_xy(cp, px0 + lp, x, y)) { pixmask[lp] = 0ull; continue; }
    PixSum ps;
    uint64_t m = 0ull;
    for (uint32_t i = 0; i < cp.spp; i++) {
      const size_t p = size_t(i) * n_pw + lp;
      ps.add(i, L[p]);
      m |= dirty[p];
    }
    pix[lp] = ps.value(cp);
    pixmask[lp] = m;
  }
}

// exclusive scan of popc(dirty) within blocks of SCAN paths; block totals to blk
__global__ void __launch_bounds__(SCAN) scan_blocks_kernel(const uint64_t* __restrict__ dirty, uint32_t P, uint32_t* __restrict__ off,
                                                           uint32_t* __restrict__ blk) {
  __shared__ uint32_t warp_tot[SCAN / 32];
  const uint32_t p = blockIdx.x * SCAN + threadIdx.x, lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  const uint32_t v = p < P ? uint32_t(__popcll(dirty[p])) : 0u;
  uint32_t inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= uint32_t(o)) inc += t;
  }
  if (lane == 31) warp_tot[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = warp_tot[lane], wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= uint32_t(o)) wi += t;
    }
    warp_tot[lane] = wi - w;   // exclusive
    if (lane == 31) blk[blockIdx.x] = wi;
  }
  __syncthreads();
  if (p < P) off[p] = warp_tot[wid] + inc - v;
}

// exclusive scan of the block totals (one block); the pair count (clamped to the pair capacity) to count_out, the
// largest total seen to status[0] and the running sum of pairs to stats[0]
__global__ void __launch_bounds__(1024) scan_top_kernel(uint32_t* __restrict__ blk, uint32_t nb, uint32_t cap, uint32_t* __restrict__ count_out,
                                                        uint32_t* __restrict__ status, unsigned long long* __restrict__ stats) {
  __shared__ uint32_t part[1024];
  const uint32_t t = threadIdx.x, per = (nb + 1023) / 1024, b0 = t * per, b1 = min(nb, b0 + per);
  uint32_t sum = 0;
  for (uint32_t b = b0; b < b1; b++) sum += blk[b];
  part[t] = sum;
  __syncthreads();
  for (uint32_t o = 1; o < 1024; o <<= 1) {
    const uint32_t v = t >= o ? part[t - o] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  uint32_t run = part[t] - sum;
  for (uint32_t b = b0; b < b1; b++) {
    const uint32_t c = blk[b];
    blk[b] = run;
    run += c;
  }
  if (t == 1023) {
    const uint32_t total = part[1023];
    *count_out = min(total, cap);
    atomicMax(status, total);
    atomicAdd(stats, (unsigned long long)total);
  }
}

// pair list: the dirty poses of path p, in increasing pose order, at pairs off[p] ...; off[p] becomes global
__global__ void __launch_bounds__(T) expand_kernel(const uint64_t* __restrict__ dirty, uint32_t P, uint32_t* __restrict__ off,
                                                   const uint32_t* __restrict__ blk, uint32_t cap, uint32_t* __restrict__ src,
                                                   uint32_t* __restrict__ pose) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const uint32_t base = off[p] + blk[p / SCAN];
    off[p] = base;
    uint64_t m = dirty[p];
    for (uint32_t j = base; m; j++, m &= m - 1ull) {
      if (j >= cap) break;
      src[j] = p;
      pose[j] = uint32_t(__ffsll((long long)m) - 1);
    }
  }
}

// every pose's value of every pixel of the wave: the shared sum where no sub-sample of the pixel is dirty for the
// pose, else the in-order sum with the re-traced radiance of its dirty sub-samples; radiance and/or raw DN out
__global__ void __launch_bounds__(T) finalize_poses_kernel(const CamParams cp, BatchView v, uint32_t px0, uint32_t n_pw, uint32_t n_poses,
                                                          BatchOut out) {
  const size_t frame = size_t(cp.w) * cp.h;
  const size_t total = size_t(n_poses) * n_pw;
  for (size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += size_t(gridDim.x) * blockDim.x) {
    const uint32_t q = uint32_t(t / n_pw), lp = uint32_t(t % n_pw);
    uint32_t x, y;
    if (!pixel_xy(cp, px0 + lp, x, y)) continue;
    float4 val;
    if (!((v.pixmask[lp] >> q) & 1ull)) {
      val = v.pix[lp];
    } else {
      PixSum ps;
      const uint64_t below = (1ull << q) - 1ull;
      for (uint32_t i = 0; i < cp.spp; i++) {
        const size_t p = size_t(i) * n_pw + lp;
        const uint64_t dm = v.dirty[p];
        float4 L;
        if ((dm >> q) & 1ull) {
          const uint32_t j = v.off[p] + uint32_t(__popcll(dm & below));
          L = j < v.cap ? v.pair_L[j] : make_float4(NAN, NAN, NAN, 0.0f);
        } else {
          L = v.shared_L[p];
        }
        ps.add(i, L);
      }
      val = ps.value(cp);
    }
    const size_t o = size_t(q) * frame + size_t(y) * cp.w + x;
    if (out.radiance) out.radiance[o] = val;
    if (out.raw && out.fused) {
      // the expose stage with no optics blur: one tap of weight 1 (gpu/wgsl/sensor.wgsl.js:177-190)
      float4 e = val;
      const float sc = out.optics_scale;
      if (sc != 1.0f) e = make_float4(__fmul_rn(e.x, sc), __fmul_rn(e.y, sc), __fmul_rn(e.z, sc), e.w);
      const float ex = __fdiv_rn(__fmaf_rn(1.0f, e.x, 0.0f), 1.0f), ey = __fdiv_rn(__fmaf_rn(1.0f, e.y, 0.0f), 1.0f),
                  ez = __fdiv_rn(__fmaf_rn(1.0f, e.z, 0.0f), 1.0f);
      out.raw[o] = uint16_t(sensor_dn(out.sensor, ex, ey, ez, int(x), int(y), int(cp.w), out.frame0 + q));
    }
  }
}
}  // namespace

void batch_camera(const Scene& S, const CamParams& cp, const BatchCull& bc, const BatchWave& bw, uint32_t n_poses, const BatchOut& out,
                  int blocks, cudaStream_t st, uint64_t* launches) {
  const uint32_t n_pix = tiled_pixels(cp.w, cp.h, cp.tile_w, cp.tile_h);
  uint64_t nl = 0;
  for (uint32_t px0 = 0; px0 < n_pix; px0 += bw.n_pw) {
    const uint32_t n_pw = std::min(bw.n_pw, n_pix - px0);
    const uint32_t P = n_pw * cp.spp;
    // shared paths
    WaveBufs ws = bw.shared;
    ws.bc = bc;
    ws.bc.dirty = bw.dirty;
    ws.bc.n_pw = n_pw;
    ws.bc.px0 = px0;
    cudaMemsetAsync(ws.counts, 0, 16, st);
    wave_gen_batch(cp, ws, blocks, st);
    wave_bounces(S, cp, ws, WAVE_SHARED, blocks, st, &nl);
    finalize_shared_kernel<<<std::max(1, std::min(blocks, int((n_pw + T - 1) / T))), T, 0, st>>>(cp, ws.L, bw.dirty, px0, n_pw, bw.pix, bw.pixmask);
    // pair list
    const uint32_t nb = (P + SCAN - 1) / SCAN;
    WaveBufs wp = bw.pairs;
    wp.bc = bc;
    wp.bc.n_pw = n_pw;
    wp.bc.px0 = px0;
    wp.bc.pair_src = bw.pair_src;
    wp.bc.pair_pose = bw.pair_pose;
    scan_blocks_kernel<<<nb, SCAN, 0, st>>>(bw.dirty, P, bw.off, bw.blk);
    scan_top_kernel<<<1, 1024, 0, st>>>(bw.blk, nb, bw.cap, wp.counts, bw.status, bw.stats);
    expand_kernel<<<blocks, T, 0, st>>>(bw.dirty, P, bw.off, bw.blk, bw.cap, bw.pair_src, bw.pair_pose);
    // pair paths
    wave_gen_pairs(cp, wp, blocks, st);
    wave_bounces(S, cp, wp, WAVE_PAIRS, blocks, st, &nl);
    BatchView v{bw.pix, bw.pixmask, bw.dirty, bw.off, ws.L, wp.L, bw.cap};
    finalize_poses_kernel<<<blocks, T, 0, st>>>(cp, v, px0, n_pw, n_poses, out);
    nl += 7;
  }
  if (launches) *launches += nl;
}

size_t batch_wave_bytes(uint32_t P, uint32_t n_pw, uint32_t cap, uint32_t n_light) {
  const size_t nb = (P + SCAN - 1) / SCAN;
  return wave_bytes(P, n_light, 0) + wave_bytes(cap, n_light, 0) + size_t(P) * 12 + nb * 4 + size_t(cap) * 8 + size_t(n_pw) * 24 + 8 * 256;
}

BatchWave batch_carve(void* base, uint32_t P, uint32_t n_pw, uint32_t cap, uint32_t n_light, uint32_t* counts, uint32_t* status,
                      unsigned long long* stats) {
  char* c = static_cast<char*>(base);
  auto take = [&](size_t bytes) { char* r = c; c += (bytes + 255) / 256 * 256; return r; };
  BatchWave b{};
  b.shared = wave_carve(take(wave_bytes(P, n_light, 0)), P, n_light, 0, counts);
  b.pairs = wave_carve(take(wave_bytes(cap, n_light, 0)), cap, n_light, 0, counts + 4);
  b.dirty = reinterpret_cast<uint64_t*>(take(size_t(P) * 8));
  b.off = reinterpret_cast<uint32_t*>(take(size_t(P) * 4));
  b.blk = reinterpret_cast<uint32_t*>(take(((P + SCAN - 1) / SCAN) * 4));
  b.pair_src = reinterpret_cast<uint32_t*>(take(size_t(cap) * 4));
  b.pair_pose = reinterpret_cast<uint32_t*>(take(size_t(cap) * 4));
  b.pix = reinterpret_cast<float4*>(take(size_t(n_pw) * 16));
  b.pixmask = reinterpret_cast<uint64_t*>(take(size_t(n_pw) * 8));
  b.status = status;
  b.stats = stats;
  b.n_pw = n_pw;
  b.cap = cap;
  return b;
}

}  // namespace vtk
