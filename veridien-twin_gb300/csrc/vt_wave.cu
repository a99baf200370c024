// Wavefront path tracing on sm_103a: the camera estimators of the twin (shadeHit, gpu/wgsl/shade.wgsl.js:250,
// and the depth-N path tracer) split into small kernels that each run one kind of work over compacted queues:
//
//   wave_gen       camera rays of a wave of sub-samples (KB4, gpu/wgsl/kernels.wgsl.js:177-185)
//   wave_extend    closest hit of every queued ray (static BVH + posed bodies)
//   wave_shade     one path vertex: emitter term, light-sample records (shadow-ray queue), BSDF continuation (next
//                  ray queue); queues are appended with one atomic per warp
//   wave_shadow    any-hit test of a path's light samples, then L += thr (sum_j visible c_j) / nL in sample order
//   wave_finalize  per pixel, the sub-samples' radiance summed in sample order (deterministic), the pixel key
//
// Path state lives in structure-of-arrays buffers in HBM (~200 B per path per bounce of traffic); the traversal
// kernels read only the ray and write only the hit, so their code and register footprint stay small and every lane
// of a warp runs the same kind of ray. The per-path arithmetic is the megakernel's: results do not depend on the
// order in which paths sit in a queue.
#include <algorithm>

#include "vt_camera.cuh"
#include "vt_wave.cuh"

namespace vtk {
using namespace vtd;

constexpr int WAVE_THREADS = 256;
// resident blocks per SM the traversal kernels are compiled for (register budget 65536 / (256 x this))
#ifndef VT_TRACE_BLOCKS
#define VT_TRACE_BLOCKS 4
#endif

// append `want` lanes' items to a queue with one atomic per warp; returns the slot of this lane (if want)
__device__ __forceinline__ uint32_t warp_append(uint32_t* count, bool want) {
  const uint32_t act = __activemask();
  const uint32_t mask = __ballot_sync(act, want);
  if (!mask) return 0;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t leader = __ffs(mask) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(count, uint32_t(__popc(mask)));
  base = __shfl_sync(act, base, leader);
  return base + __popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ void init_path(const WaveBufs& wb, uint32_t p, float4 o4, float4 d4, uint32_t id, uint32_t i, uint32_t hs, bool valid) {
  wb.o[p] = o4;
  wb.d[p] = d4;
  wb.thr[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
  wb.L[p] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0xfffeu));
  wb.meta[p] = make_uint4(id, i, hs, valid ? 1u : 0u);      // bounce 1 (0: no pixel)
}

// the scene a path sees: its pose's uniform for a pair path, the shared one otherwise
template <int VAR>
__device__ __forceinline__ Scene path_scene(const Scene& S, const WaveBufs& wb, uint32_t p) {
  if (VAR != WAVE_PAIRS) return S;
  Scene s = S;
  s.su = wb.bc.su_base + size_t(__ldg(wb.bc.pair_pose + p)) * wb.bc.su_stride;
  return s;
}

// The poses of a batch whose copy of a varying body the segment o + t d, t in [0, t1], may reach: the world-box and
// capsule culls that trace_scene applies to a body before traversing it (gpu/wgsl/trace.wgsl.js:302), with a relative
// margin, over the batch's BVH of (pose, body) items. A pose not returned cannot change the segment's result, so
// the returned set is a superset of the poses whose traced result differs from the shared one; on any overflow
// every pose is returned.
__device__ __forceinline__ uint64_t cull_bits(const BatchCull& C, float3 o, float3 d, float t1, uint32_t skip, uint64_t have) {
  if (!C.n_nodes) return 0ull;
  const float te = t1 < BIG ? t1 + fabsf(t1) * 1e-5f + 1e-6f : BIG;
  const float tc = fminf(te, 1e3f);
  const float3 inv = safe_inv(d);
  uint64_t bits = 0ull;
  constexpr int DEPTH = 24;
  uint32_t stack[DEPTH];
  int sp = 0;
  uint32_t n = 0;
  for (uint32_t guard = 0;; guard++) {
    if (guard > 2u * C.n_nodes + 2u) return ~0ull;
    const float4 a = __ldg(C.nodes + 2u * n), b = __ldg(C.nodes + 2u * n + 1u);
    const uint32_t ref = __float_as_uint(a.w), cnt = __float_as_uint(b.w);
    if (slab(xyz(a), xyz(b), o, inv, 0.0f, te) < BIG) {
      if (cnt == 0u) {
        if (sp >= DEPTH) return ~0ull;
        stack[sp++] = ref + 1u;
        n = ref;
        continue;
      }
      for (uint32_t k = 0; k < cnt; k++) {
        const float4* it = C.items + 4u * (ref + k);
        const float4 lo = __ldg(it), hi = __ldg(it + 1);
        const uint32_t q = __float_as_uint(lo.w), body = __float_as_uint(hi.w);
        if ((((have | bits) >> q) & 1ull) || ((skip >> body) & 1u)) continue;
        if (slab(xyz(lo), xyz(hi), o, inv, 0.0f, te) >= BIG) continue;
        const float4 ca = __ldg(it + 2), cb = __ldg(it + 3);
        if (seg_near_capsule(o, d, 0.0f, tc, xyz(ca), xyz(cb), ca.w * 1.001f + 1e-5f)) bits |= 1ull << q;
      }
    }
    if (!sp) break;
    n = stack[--sp];
  }
  return bits;
}

// paths of the wave: sub-sample index i in [i0, i0 + n_i), pixel id in [0, n_pix); path p = (i - i0) * n_pix + id
__global__ void __launch_bounds__(WAVE_THREADS) wave_gen(const CamParams cp, WaveBufs wb, uint32_t i0, uint32_t n_i, uint32_t n_pix) {
  const uint32_t total = n_i * n_pix;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
    const uint32_t id = p % n_pix, i = i0 + p / n_pix;
    float4 o4, d4;
    uint32_t hs;
    const bool valid = camera_path(cp, id, i, o4, d4, hs);
    init_path(wb, p, o4, d4, id, i, hs, valid);
    const uint32_t slot = warp_append(wb.count_in, valid);
    if (valid) wb.q_in[slot] = p;
  }
}

// a batch wave: paths p = i * n_pw + lp (all sub-samples i < spp of pixels px0 + lp)
__global__ void __launch_bounds__(WAVE_THREADS) wave_gen_batch_kernel(const CamParams cp, WaveBufs wb) {
  const uint32_t n_pw = wb.bc.n_pw, total = cp.spp * n_pw;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
    const uint32_t id = wb.bc.px0 + p % n_pw, i = p / n_pw;
    float4 o4, d4;
    uint32_t hs;
    const bool valid = camera_path(cp, id, i, o4, d4, hs);
    init_path(wb, p, o4, d4, id, i, hs, valid);
    wb.bc.dirty[p] = 0ull;
    const uint32_t slot = warp_append(wb.count_in, valid);
    if (valid) wb.q_in[slot] = p;
  }
}

// pair paths: pair j repeats shared path pair_src[j] (same pixel and sub-sample) under its own pose
__global__ void __launch_bounds__(WAVE_THREADS) wave_gen_pairs_kernel(const CamParams cp, WaveBufs wb) {
  const uint32_t n = *wb.count_in, n_pw = wb.bc.n_pw;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const uint32_t p = wb.bc.pair_src[j];
    const uint32_t id = wb.bc.px0 + p % n_pw, i = p / n_pw;
    float4 o4, d4;
    uint32_t hs;
    const bool valid = camera_path(cp, id, i, o4, d4, hs);
    init_path(wb, j, o4, d4, id, i, hs, valid);
    wb.q_in[j] = j;
  }
}

// HC: the static first-hit cache is on (compiled separately, so the plain kernel keeps its registers)
template <int VAR, bool HC = false>
__global__ void __launch_bounds__(WAVE_THREADS, VT_TRACE_BLOCKS) wave_extend(const Scene S, const CamParams cp, WaveBufs wb) {
  const uint32_t n = *wb.count_in;
  if (wb.stats && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(wb.stats, (unsigned long long)n);
  __shared__ uint2 stack_sh[SH_DEPTH * WAVE_THREADS];
  __shared__ float4 top_sh[4u * (TOP_NODES ? TOP_NODES : 1u)];
  LaneStack stk;
  stk.sh = stack_sh; stk.lane = threadIdx.x; stk.stride = WAVE_THREADS; stk.top = top_sh;
  TraceState st;
  const uint32_t root = stage_top(S, top_sh, cp.root);
  Scene Sl = S;
  float3 o = f3(0, 0, 0), d = f3(0, 0, 1);
  float tt = 0.0f;
  uint32_t p = 0, skip = 0;
  bool active = false, exhausted = false;
  auto finish = [&]() {
    wb.hit[p] = make_float4(st.best.t, st.best.u, st.best.v, __uint_as_float(st.best.tri));
    wb.hinst[p] = st.best.inst;
    if (VAR == WAVE_SHARED) {
      const uint64_t have = wb.bc.dirty[p];
      const uint64_t bits = cull_bits(wb.bc, o, d, st.best.t, skip, have);
      if (bits & ~have) wb.bc.dirty[p] = have | bits;
    }
    active = false;
  };
  // static first-hit cache (camera rays of a fixed camera, gpu/wgsl/kernels.wgsl.js:82 staticFirstHit): a cached
  // entry replaces the static phase (the instance phases then start from it, exactly as after tracing it); an empty
  // one is filled when the static phase ends
  uint32_t ci = MISS;
  auto start = [&](uint32_t idx) {
    p = wb.q_in[idx];
    const float4 o4 = wb.o[p], d4 = wb.d[p];
    o = xyz(o4); d = xyz(d4); tt = o4.w;
    const uint4 meta = wb.meta[p];
    skip = meta.w == 1 ? cp.skip : 0u;
    Sl = path_scene<VAR>(S, wb, p);
    st.best = Hit{BIG, 0.0f, 0.0f, MISS, MISS};
    int from = -1;
    ci = MISS;
    if (HC && VAR == WAVE_PLAIN && meta.w == 1 && meta.y < wb.hc_cap) {
      ci = meta.y * wb.hc_stride + meta.x;
      const float4 h = wb.hcache[ci];
      if (h.x > 0.0f) { st.best = Hit{h.x, h.y, h.z, __float_as_uint(h.w), MISS}; from = 0; ci = MISS; }
    }
    active = trace_phase(Sl, root, o, d, 0.0f, tt, 3u, VAR == WAVE_SHARED ? (skip | wb.bc.vary) : skip, st, from);
    if (HC && ci != MISS && st.k != -1) {   // no static phase to wait for: the static hit is none
      wb.hcache[ci] = make_float4(BIG, 0.0f, 0.0f, __uint_as_float(MISS));
      ci = MISS;
    }
    if (!active) { active = true; finish(); }
  };
  while (take_rays(active, exhausted, wb.fetch, n, cp.refill, start)) {
    if (!active) continue;
    const int r = trace_step<false>(Sl, 0.0f, st, stk);
    if (HC && r != 0 && VAR == WAVE_PLAIN && ci != MISS && st.k == -1) {
      wb.hcache[ci] = make_float4(st.best.t, st.best.u, st.best.v, __uint_as_float(st.best.tri));
      ci = MISS;
    }
    if (r != 0 && !trace_phase(Sl, root, o, d, 0.0f, tt, 3u, VAR == WAVE_SHARED ? (skip | wb.bc.vary) : skip, st, st.k + 1)) finish();
  }
}

template <int MODE, int VAR>
// blocks of 256 an SM holds: 3 caps the registers at 80 (the compiler takes 142 uncapped, one block per SM). C0
// (640x480, 16 spp, depth 4): 24.35 ms at 1 block, 21.93 at 2 (100 registers), 21.30 at 3, 21.37 at 4; images
// identical
#ifndef VT_WAVE_SHADE_BLOCKS
#define VT_WAVE_SHADE_BLOCKS 3
#endif
__global__ void __launch_bounds__(WAVE_THREADS, VT_WAVE_SHADE_BLOCKS) wave_shade(const Scene S0, const CamParams cp, WaveBufs wb) {
  const uint32_t n = *wb.count_in;
  const uint32_t nl = cp.n_light;
  const bool no_mis = (cp.options & VT_O_NO_MIS) != 0u;
  const float emit_area = __ldg(S0.su + 3);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const uint32_t p = wb.q_in[k];
    const Scene S = path_scene<VAR>(S0, wb, p);
    const uint4 meta = wb.meta[p];
    const uint32_t i = meta.y, hs = meta.z, b = meta.w;
    const float4 o4 = wb.o[p], d4 = wb.d[p], hv = wb.hit[p];
    float4 L4 = wb.L[p];
    float3 L = xyz(L4), thr = xyz(wb.thr[p]);
    const float3 o = xyz(o4), d = xyz(d4);
    const float tt = o4.w, pdf_prev = d4.w;
    Hit h{hv.x, hv.y, hv.z, __float_as_uint(hv.w), wb.hinst[p]};
    bool cont = false, shadow = false;
    if (h.tri != MISS) {
      const Surf s = surface(S, h, o, d, tt);
      const float3 wo = -d;
      const bool is_static = (s.flags & VT_F_STATIC) != 0u;
      if (b == 1) L4.w = __uint_as_float(s.mesh | ((h.inst == MISS || is_static) ? 0u : 0x10000u));
      if (MODE == VT_SHADE_TWIN && b == 2) {
        // gpu/wgsl/shade.wgsl.js:224 secondary
        if (s.flags & VT_F_EMITTER) {
          if (!no_mis) {
            const float3 nE = emitter_normal(S, h, s, tt);
            const float cosE = dot(-d, nE);
            if (cosE > 0.0f) {
              const float3 Le = emitted(S, nE, emitter_axis_at(S, tt), -d);
              const float pdfL = h.t * h.t / (cosE * emit_area);
              L = L + thr * (Le * (pdf_prev * pdf_prev / (pdf_prev * pdf_prev + float(nl) * float(nl) * pdfL * pdfL)));
            }
          }
        } else if (!(cp.options & (VT_O_DIRECT_ONLY | VT_O_NO_INDIRECT))) {
          if (is_static) {
            const uint32_t slot = ldu(S.su + 18);
            L = L + thr * (albedo(S, s.mat, clampf(dot(s.ns, -d), 0.0f, 1.0f)) * node_slot(S, s, slot, slot));
          } else {
            const Mat M2 = load_mat(S, s.mat);
            L = L + thr * (M2.hh * ld3(S.su + 8) * INV_PI_F);
          }
        }
      } else if (MODE == VT_SHADE_TWIN && (cp.options & VT_O_NORMALS)) {
        L = s.ns * 0.5f + f3(0.5f, 0.5f, 0.5f);
      } else if (s.flags & VT_F_EMITTER) {
        const float3 nE = emitter_normal(S, h, s, tt);
        const float3 Le = emitted(S, nE, emitter_axis_at(S, tt), wo);
        if (b == 1) {
          L = L + thr * Le;
        } else if (!no_mis) {
          const float cosE = dot(-d, nE);
          if (cosE > 0.0f) {
            const float pdfL = h.t * h.t / (cosE * emit_area);
            L = L + thr * Le * (pdf_prev * pdf_prev / (pdf_prev * pdf_prev + float(nl) * float(nl) * pdfL * pdfL));
          }
        }
      } else {
        const Mat M = load_mat(S, s.mat);
        const float3 n = shading_normal(S, s, cp.options);
        const bool mis = !no_mis && (MODE == VT_SHADE_PATH || !is_static);
        const float sh0 = b == 1 ? u01(pcg(hs + 3u)) : bounce_shift(hs, b, 0);
        const float sh1 = b == 1 ? u01(pcg(hs + 4u)) : bounce_shift(hs, b, 1);
        const float sh2 = b == 1 ? u01(pcg(hs + 5u)) : bounce_shift(hs, b, 2);
        // nL emitter samples: the unshadowed contribution and the shadow segment of each (shade.wgsl.js:135 lightEval).
        // The record's flag: 0 no contribution, 1 trace it (static scene and posed bodies); with the static-occlusion
        // cache (a static first hit, shade.wgsl.js:270-301): 4 trace the static scene (its answer fills the cache) then
        // the bodies, 5 the static scene is known clear (trace the bodies), 6 the static scene is known to hide it
        const bool cached = MODE == VT_SHADE_TWIN && VAR == WAVE_PLAIN && b == 1 && is_static && wb.scache && i < wb.hc_cap;
        uint32_t word = 0;
        if (cached) word = wb.scache[i * wb.hc_stride + meta.x];
        float4* rec = wb.sh + size_t(p) * nl * 3;
        uint32_t nlit = 0;
        for (uint32_t j = 0; j < nl; j++) {
          const float3 u = f3(kr(i * nl + j, KL0, sh0), kr(i * nl + j, KL1, sh1), kr(i * nl + j, KL2, sh2));
          float3 c, so, wi;
          float tmax;
          const bool ok = light_sample(S, s, n, M, wo, tt, u, mis, float(nl), c, so, wi, tmax);
          float flag = ok ? 1.0f : 0.0f;
          if (cached && ok) flag = (word >> 31) ? (((word >> j) & 1u) ? 6.0f : 5.0f) : 4.0f;
          rec[3 * j] = make_float4(so.x, so.y, so.z, tmax);
          rec[3 * j + 1] = make_float4(wi.x, wi.y, wi.z, flag);
          rec[3 * j + 2] = make_float4(c.x, c.y, c.z, 0.0f);
          nlit += ok ? 1u : 0u;
          shadow |= ok && flag != 6.0f;
        }
        if (cached) {
          rec[2].w = __uint_as_float(nlit);   // the shadow kernel's penumbra test needs the lit count
          if (!(word >> 31) && nlit == 0) wb.scache[i * wb.hc_stride + meta.x] = 0x80000000u;
        }
        if (shadow) wb.nee[p] = make_float4(thr.x, thr.y, thr.z, tt);
        // key bit 0x20000: a first-hit light sample needs its shadow ray (shade.wgsl.js:177, no shadow culling); with
        // the static-occlusion cache the shadow kernel decides it (a body blocks a sample, a penumbra, uneven samples)
        if (b == 1 && shadow && !cached) L4.w = __uint_as_float(__float_as_uint(L4.w) | 0x20000u);
        bool bounce;
        if (MODE == VT_SHADE_TWIN) {
          bounce = !is_static;
          if (is_static && !(cp.options & (VT_O_NO_INDIRECT | VT_O_DIRECT_ONLY))) {
            float3 E = node_slot(S, s, 0u, ldu(S.su + 18));
            if (!(cp.options & VT_O_NO_CAPSULE)) E = E * capsule_vis(S, s.p, n);
            L = L + E * INV_PI_F * albedo(S, s.mat, fmaxf(dot(n, wo), 0.0f));
          }
        } else {
          bounce = b < cp.max_depth;
        }
        if (bounce) {
          const float3 ub = b == 1 ? f3(kr(i, KB0, u01(pcg(hs + 6u))), kr(i, KB1, u01(pcg(hs + 7u))), kr(i, KB2, u01(pcg(hs + 8u))))
                                   : f3(kr(i, KB0, bounce_shift(hs, b, 3)), kr(i, KB1, bounce_shift(hs, b, 4)), kr(i, KB2, bounce_shift(hs, b, 5)));
          float3 l;
          const float pdf = sample_bsdf(M, n, wo, ub, l);
          if (pdf > 0.0f && dot(s.ng, l) > 0.0f) {
            thr = thr * eval_bsdf(M, n, l, wo) * (dot(n, l) / pdf);
            const float3 no = offset_ray(s.p, s.ng, l);
            wb.o[p] = make_float4(no.x, no.y, no.z, tt);
            wb.d[p] = make_float4(l.x, l.y, l.z, pdf);
            wb.thr[p] = make_float4(thr.x, thr.y, thr.z, 0.0f);
            wb.meta[p] = make_uint4(meta.x, meta.y, meta.z, b + 1u);
            cont = true;
          }
        }
      }
    }
    wb.L[p] = make_float4(L.x, L.y, L.z, L4.w);
    const uint32_t qs = warp_append(wb.count_out, cont);
    if (cont) wb.q_out[qs] = p;
    const uint32_t ss = warp_append(wb.count_sh, shadow);
    if (shadow) wb.q_sh[ss] = p;
  }
}

// any-hit of every queued path's light samples in sample order on persistent lanes; a lane moves to the path's next
// sample when one finishes, and to a new path when the last one does
// SC: the static-occlusion cache is on (compiled separately, so the plain kernel keeps its registers)
template <int VAR, bool SC = false>
__global__ void __launch_bounds__(WAVE_THREADS, VT_TRACE_BLOCKS) wave_shadow(const Scene S0, const CamParams cp, WaveBufs wb) {
  const uint32_t n = *wb.count_sh;
  if (wb.stats && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(wb.stats + 1, (unsigned long long)n);
  const uint32_t nl = cp.n_light;
  const uint32_t skip0 = ldu(S0.su + 7);
  const uint32_t skip = VAR == WAVE_SHARED ? (skip0 | wb.bc.vary) : skip0;
  __shared__ uint2 stack_sh[SH_DEPTH * WAVE_THREADS];
  __shared__ float4 top_sh[4u * (TOP_NODES ? TOP_NODES : 1u)];
  LaneStack stk;
  stk.sh = stack_sh; stk.lane = threadIdx.x; stk.stride = WAVE_THREADS; stk.top = top_sh;
  TraceState st;
  const uint32_t root = stage_top(S0, top_sh, cp.root);
  Scene S = S0;
  float3 o = f3(0, 0, 0), d = f3(0, 0, 1);
  float4 nee = make_float4(0, 0, 0, 0);
  float3 Ld = f3(0, 0, 0);
  uint32_t p = 0, j = 0;
  uint64_t have = 0ull, bits = 0ull;
  bool active = false, exhausted = false;
  const float4* rec = nullptr;
  // the static-occlusion cache's bookkeeping of the current path (shade.wgsl.js:270-301): lit and visible samples,
  // their luminance range, a posed body blocking one, and the occlusion word to store
  bool cm = false, dyn = false, fill = false;
  uint32_t nvis = 0, nlit = 0, word = 0, ci = 0;
  float lmin = BIG, lmax = 0.0f;
  auto visible = [&](uint32_t jj) {
    const float3 c = xyz(rec[3 * jj + 2]);
    Ld = Ld + c;
    if (SC && cm) {
      nvis++;
      const float y = lum(c);
      lmin = fminf(lmin, y);
      lmax = fmaxf(lmax, y);
    }
  };
  // the next light sample of the path with a valid record at or after j, set up as a ray; false when none is left
  auto next_sample = [&]() -> bool {
    for (; j < nl; j++) {
      const float4 a = rec[3 * j], w = rec[3 * j + 1];
      if (w.w == 0.0f || (SC && w.w == 6.0f)) continue;   // no contribution, or hidden by the static scene (cached)
      o = xyz(a); d = xyz(w);
      st.best = Hit{a.w, 0.0f, 0.0f, MISS, MISS};
      if (trace_phase(S, root, o, d, 0.0f, nee.w, 3u, skip, st, SC && w.w == 5.0f ? 0 : -1)) return true;
      // nothing to traverse: the segment is unoccluded
      visible(j);
      if (VAR == WAVE_SHARED) bits |= cull_bits(wb.bc, o, d, a.w, skip0, have | bits);
    }
    return false;
  };
  auto finish_path = [&]() {
    const float4 L = wb.L[p];
    const float3 v = xyz(L) + xyz(nee) * (Ld / float(nl));
    uint32_t key = __float_as_uint(L.w);
    if (SC && cm) {
      if (fill) wb.scache[ci] = word | 0x80000000u;
      if (dyn || (nvis > 0u && nvis < nlit) || (nvis > 1u && lmax - lmin > 0.2f * (lmax + lmin) * 0.5f)) key |= 0x20000u;
    }
    wb.L[p] = make_float4(v.x, v.y, v.z, __uint_as_float(key));
    if (VAR == WAVE_SHARED && bits) wb.bc.dirty[p] = have | bits;
    active = false;
  };
  auto start = [&](uint32_t idx) {
    p = wb.q_sh[idx];
    S = path_scene<VAR>(S0, wb, p);
    nee = wb.nee[p];
    rec = wb.sh + size_t(p) * nl * 3;
    Ld = f3(0, 0, 0);
    j = 0;
    bits = 0ull;
    if (VAR == WAVE_SHARED) have = wb.bc.dirty[p];
    cm = fill = dyn = false;
    if (SC && VAR == WAVE_PLAIN) {
      for (uint32_t q = 0; q < nl; q++) {
        const float f = rec[3 * q + 1].w;
        cm |= f >= 4.0f;
        fill |= f == 4.0f;
      }
      if (cm) {
        const uint4 meta = wb.meta[p];
        ci = meta.y * wb.hc_stride + meta.x;
        nlit = __float_as_uint(rec[2].w);
        nvis = 0;
        word = 0;
        lmin = BIG;
        lmax = 0.0f;
      }
    }
    active = true;
    if (!next_sample()) finish_path();
  };
  while (take_rays(active, exhausted, wb.fetch, n, cp.refill, start)) {
    if (!active) continue;
    const int r = trace_step<true>(S, 0.0f, st, stk);
    bool done = r == 2;
    if (r == 1) done = !trace_phase(S, root, o, d, 0.0f, nee.w, 3u, skip, st, st.k + 1);
    if (!done) continue;
    if (st.best.tri == MISS) {
      visible(j);
      if (VAR == WAVE_SHARED) bits |= cull_bits(wb.bc, o, d, rec[3 * j].w, skip0, have | bits);
    } else if (SC && cm) {
      if (st.k < 0) word |= 1u << j;   // the static scene hides it
      else dyn = true;                 // a posed body does
    }
    j++;
    if (!next_sample()) finish_path();
  }
}

// per pixel, the wave's sub-samples in order i0..i0+n_i-1 added to the running sum; the last wave writes the pixel
__global__ void __launch_bounds__(WAVE_THREADS) wave_finalize(const CamParams cp, WaveBufs wb, uint32_t i0, uint32_t n_i, uint32_t n_pix,
                                                             float4* __restrict__ acc, float4* __restrict__ out, int last) {
  for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n_pix; id += gridDim.x * blockDim.x) {
    uint32_t x, y;
    if (!pixel_xy(cp, id, x, y)) continue;
    float4 a = i0 == 0 ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : acc[id];
    float3 s = xyz(a);
    uint32_t key = __float_as_uint(a.w);
    for (uint32_t k = 0; k < n_i; k++) {
      const float4 L = wb.L[size_t(k) * n_pix + id];
      s = s + xyz(L);
      const uint32_t gk = __float_as_uint(L.w);
      if (i0 + k == 0) key = gk;
      else if ((gk & 0xffffu) != (key & 0xffffu)) key |= 0x40000u;
      key |= gk & 0x30000u;
    }
    if (last) {
      const float sc = cp.scale / float(cp.spp);
      out[size_t(y) * cp.w + x] = make_float4(s.x * sc, s.y * sc, s.z * sc, key == 0xfffeu ? 0.0f : 1.0f);
    } else {
      acc[id] = make_float4(s.x, s.y, s.z, __uint_as_float(key));
    }
  }
}

// ------------------------------------------------------------------------------------------------ refinement
// gpu/wgsl/kernels.wgsl.js:218 camRefine: after pass 1, a pixel whose sub-samples saw different meshes (key bit
// 0x40000), a posed body (0x10000), a shadow-traced pixel when VT_O_REFINE_SHADOW is set (0x20000), or whose 3x3
// neighbourhood has another first-hit mesh gets cp.refine more sub-samples (indices spp .. spp + refine - 1, the same
// sequences), added in order to its pass-1 sum: value = sum * scale / (spp + refine), alpha 1. The others keep the
// pass-1 value. Refined pixels are counted into dbg[2..5] (total, posed body, shadow, sub-sample mesh change).
__device__ __forceinline__ uint32_t pixel_id(const CamParams& cp, uint32_t x, uint32_t y) {
  const uint32_t tw = cp.tile_w, th = cp.tile_h, tiles_x = (cp.w + tw - 1) / tw;
  return ((y / th) * tiles_x + x / tw) * (tw * th) + (y % th) * tw + (x % tw);
}

__global__ void __launch_bounds__(WAVE_THREADS) refine_select(const CamParams cp, const Scene S, WaveBufs wb, uint32_t n_pix, float4* __restrict__ out) {
  for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n_pix; id += gridDim.x * blockDim.x) {
    uint32_t x, y;
    bool want = false;
    if (pixel_xy(cp, id, x, y)) {
      const float4 a = wb.acc[id];
      const uint32_t k = __float_as_uint(a.w);
      want = (k & 0x50000u) != 0u || ((k & 0x20000u) != 0u && (cp.options & VT_O_REFINE_SHADOW) != 0u);
      for (int dy = -1; dy <= 1 && !want; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          const uint32_t xx = uint32_t(min(max(int(x) + dx, 0), int(cp.w) - 1)), yy = uint32_t(min(max(int(y) + dy, 0), int(cp.h) - 1));
          if ((__float_as_uint(wb.acc[pixel_id(cp, xx, yy)].w) & 0xffffu) != (k & 0xffffu)) { want = true; break; }
        }
      if (want) {
        atomicAdd(S.dbg + 2, 1u);
        if (k & 0x10000u) atomicAdd(S.dbg + 3, 1u);
        if (k & 0x20000u) atomicAdd(S.dbg + 4, 1u);
        if (k & 0x40000u) atomicAdd(S.dbg + 5, 1u);
      } else {
        const float sc = cp.scale / float(cp.spp);
        out[size_t(y) * cp.w + x] = make_float4(a.x * sc, a.y * sc, a.z * sc, k == 0xfffeu ? 0.0f : 1.0f);
      }
    }
    const uint32_t slot = warp_append(wb.rcount, want);
    if (want) wb.rlist[slot] = id;
  }
}

// refinement paths p = e * n_list + l: sub-sample spp + e0 + e of listed pixel l
__global__ void __launch_bounds__(WAVE_THREADS) refine_gen(const CamParams cp, WaveBufs wb, uint32_t spp1, uint32_t e0, uint32_t n_e) {
  const uint32_t n_list = *wb.rcount, total = n_list * n_e;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
    const uint32_t l = p % n_list, i = spp1 + e0 + p / n_list, id = wb.rlist[l];
    float4 o4, d4;
    uint32_t hs;
    const bool valid = camera_path(cp, id, i, o4, d4, hs);
    init_path(wb, p, o4, d4, id, i, hs, valid);
    const uint32_t slot = warp_append(wb.count_in, valid);
    if (valid) wb.q_in[slot] = p;
  }
}

__global__ void __launch_bounds__(WAVE_THREADS) refine_finalize(const CamParams cp, WaveBufs wb, uint32_t spp1, uint32_t e0, uint32_t n_e,
                                                               float4* __restrict__ out, int last) {
  const uint32_t n_list = *wb.rcount;
  for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < n_list; l += gridDim.x * blockDim.x) {
    const uint32_t id = wb.rlist[l];
    float3 s = xyz(e0 == 0 ? wb.acc[id] : wb.acc2[l]);
    for (uint32_t e = 0; e < n_e; e++) s = s + xyz(wb.L[size_t(e) * n_list + l]);
    if (last) {
      uint32_t x, y;
      pixel_xy(cp, id, x, y);
      const float sc = cp.scale / float(spp1 + cp.refine);
      out[size_t(y) * cp.w + x] = make_float4(s.x * sc, s.y * sc, s.z * sc, 1.0f);
    } else {
      wb.acc2[l] = make_float4(s.x, s.y, s.z, 0.0f);
    }
  }
}

size_t wave_bytes(uint32_t paths, uint32_t n_light, uint32_t n_pix) {
  const size_t P = paths;
  return P * (16 * 7 + 4 * 4) + P * size_t(n_light) * 48 + size_t(n_pix) * 36 + 18 * 256;
}

WaveBufs wave_carve(void* base, uint32_t paths, uint32_t n_light, uint32_t n_pix, uint32_t* counts) {
  char* c = static_cast<char*>(base);
  auto take = [&](size_t bytes) { char* r = c; c += (bytes + 255) / 256 * 256; return r; };
  const size_t P = paths;
  WaveBufs w{};
  w.o = reinterpret_cast<float4*>(take(P * 16));
  w.d = reinterpret_cast<float4*>(take(P * 16));
  w.thr = reinterpret_cast<float4*>(take(P * 16));
  w.L = reinterpret_cast<float4*>(take(P * 16));
  w.hit = reinterpret_cast<float4*>(take(P * 16));
  w.nee = reinterpret_cast<float4*>(take(P * 16));
  w.meta = reinterpret_cast<uint4*>(take(P * 16));
  w.hinst = reinterpret_cast<uint32_t*>(take(P * 4));
  w.qa = reinterpret_cast<uint32_t*>(take(P * 4));
  w.qb = reinterpret_cast<uint32_t*>(take(P * 4));
  w.q_sh = reinterpret_cast<uint32_t*>(take(P * 4));
  w.sh = reinterpret_cast<float4*>(take(P * size_t(n_light) * 48));
  w.acc = reinterpret_cast<float4*>(take(size_t(n_pix) * 16));
  w.acc2 = reinterpret_cast<float4*>(take(size_t(n_pix) * 16));
  w.rlist = reinterpret_cast<uint32_t*>(take(size_t(n_pix) * 4));
  w.rcount = nullptr;
  w.hcache = nullptr;
  w.scache = nullptr;
  w.hc_stride = w.hc_cap = 0;
  w.counts = counts;
  w.fetch = counts + 3;
  return w;
}

// event pair around one launch when a timer has room
struct TimedLaunch {
  KernelTimer* t;
  cudaStream_t st;
  int slot = -1;
  TimedLaunch(KernelTimer* t_, cudaStream_t s, uint8_t kind) : t(t_), st(s) {
    if (t && t->n + 1 <= t->cap) { slot = t->n++; t->kind[slot] = kind; cudaEventRecord(t->ev[2 * slot], st); }
  }
  ~TimedLaunch() { if (slot >= 0) cudaEventRecord(t->ev[2 * slot + 1], st); }
};

// wave_shade's grid-stride loop over the queue runs in VT_WAVE_SHADE_WAVES waves of its own occupancy (the
// traversal kernels' grid is sized for theirs); 1, 2 and 4 waves measured within 0.2 % on C0
#ifndef VT_WAVE_SHADE_WAVES
#define VT_WAVE_SHADE_WAVES 1
#endif
template <int MODE, int VAR>
int shade_grid() {
  static std::atomic<int> grid[MAX_DEVICES];
  return per_device_value(grid, [](int dev) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, wave_shade<MODE, VAR>, WAVE_THREADS, 0);
    return device_sms(dev) * std::max(1, per) * VT_WAVE_SHADE_WAVES;
  });
}

template <int VAR>
void bounce_kernels(const Scene& S, const CamParams& cp, const WaveBufs& w, int blocks, cudaStream_t st, KernelTimer* timer) {
  cudaMemsetAsync(w.fetch, 0, 4, st);
  {
    TimedLaunch tl(timer, st, 0);
    if (VAR == WAVE_PLAIN && w.hcache) wave_extend<VAR, true><<<blocks, WAVE_THREADS, 0, st>>>(S, cp, w);
    else wave_extend<VAR, false><<<blocks, WAVE_THREADS, 0, st>>>(S, cp, w);
  }
  {
    TimedLaunch tl(timer, st, 1);
    if (cp.mode == VT_SHADE_TWIN) wave_shade<VT_SHADE_TWIN, VAR><<<shade_grid<VT_SHADE_TWIN, VAR>(), WAVE_THREADS, 0, st>>>(S, cp, w);
    else wave_shade<VT_SHADE_PATH, VAR><<<shade_grid<VT_SHADE_PATH, VAR>(), WAVE_THREADS, 0, st>>>(S, cp, w);
  }
  cudaMemsetAsync(w.fetch, 0, 4, st);
  {
    TimedLaunch tl(timer, st, 2);
    if (VAR == WAVE_PLAIN && w.scache) wave_shadow<VAR, true><<<blocks, WAVE_THREADS, 0, st>>>(S, cp, w);
    else wave_shadow<VAR, false><<<blocks, WAVE_THREADS, 0, st>>>(S, cp, w);
  }
}

void wave_bounces(const Scene& S, const CamParams& cp, WaveBufs wb, int var, int blocks, cudaStream_t st, uint64_t* launches, KernelTimer* timer) {
  const uint32_t depth = cp.mode == VT_SHADE_TWIN ? 2u : cp.max_depth;
  WaveBufs w = wb;
  for (uint32_t b = 1; b <= depth; b++) {
    // queue of this bounce in (qa | qb), next bounce's in the other; counters 0/1 alternate, 2 is the shadow count
    w.q_in = (b & 1) ? wb.qa : wb.qb;
    w.q_out = (b & 1) ? wb.qb : wb.qa;
    w.count_in = wb.counts + ((b & 1) ? 0 : 1);
    w.count_out = wb.counts + ((b & 1) ? 1 : 0);
    w.count_sh = wb.counts + 2;
    cudaMemsetAsync(w.count_out, 0, 4, st);
    cudaMemsetAsync(w.count_sh, 0, 4, st);
    if (var == WAVE_SHARED) bounce_kernels<WAVE_SHARED>(S, cp, w, blocks, st, timer);
    else if (var == WAVE_PAIRS) bounce_kernels<WAVE_PAIRS>(S, cp, w, blocks, st, timer);
    else bounce_kernels<WAVE_PLAIN>(S, cp, w, blocks, st, timer);
    if (launches) *launches += 3;
  }
}

void launch_wave_extend(const Scene& S, const CamParams& cp, const WaveBufs& wb, int blocks, cudaStream_t st) {
  cudaMemsetAsync(wb.fetch, 0, 4, st);
  wave_extend<WAVE_PLAIN, false><<<blocks, WAVE_THREADS, 0, st>>>(S, cp, wb);
}

void launch_wave_gen(const CamParams& cp, WaveBufs wb, uint32_t i0, uint32_t n_i, uint32_t n_pix, int blocks, cudaStream_t st) {
  wb.q_in = wb.qa;
  wb.count_in = wb.counts;
  wave_gen<<<blocks, WAVE_THREADS, 0, st>>>(cp, wb, i0, n_i, n_pix);
}

void wave_gen_batch(const CamParams& cp, WaveBufs wb, int blocks, cudaStream_t st) {
  wb.q_in = wb.qa;
  wb.count_in = wb.counts;
  wave_gen_batch_kernel<<<blocks, WAVE_THREADS, 0, st>>>(cp, wb);
}

void wave_gen_pairs(const CamParams& cp, WaveBufs wb, int blocks, cudaStream_t st) {
  wb.q_in = wb.qa;
  wb.count_in = wb.counts;
  wave_gen_pairs_kernel<<<blocks, WAVE_THREADS, 0, st>>>(cp, wb);
}

// one camera: waves of whole sub-sample indices, each bounce extend -> shade -> shadow over compacted queues
void wave_render(const Scene& S, const CamParams& cp, WaveBufs wb, uint32_t wave_paths, float4* out, int blocks, cudaStream_t st,
                 uint64_t* launches, KernelTimer* timer, const CamParams* cp2) {
  const uint32_t n_pix = tiled_pixels(cp.w, cp.h, cp.tile_w, cp.tile_h);
  const uint32_t per_wave = std::max(1u, std::min(cp.spp, wave_paths / n_pix));
  uint64_t nlaunch = 0;
  for (uint32_t i0 = 0; i0 < cp.spp; i0 += per_wave) {
    const uint32_t n_i = std::min(per_wave, cp.spp - i0);
    cudaMemsetAsync(wb.counts, 0, 16, st);
    WaveBufs w = wb;
    w.q_in = wb.qa; w.count_in = wb.counts + 0;
    wave_gen<<<blocks, WAVE_THREADS, 0, st>>>(cp, w, i0, n_i, n_pix);
    nlaunch++;
    wave_bounces(S, cp, wb, WAVE_PLAIN, blocks, st, &nlaunch, timer);
    const int last = i0 + n_i >= cp.spp && !(cp.refine && cp2 && wb.rcount);
    wave_finalize<<<blocks, WAVE_THREADS, 0, st>>>(cp, wb, i0, n_i, n_pix, wb.acc, out, last);
    nlaunch++;
  }
  if (cp.refine && cp2 && wb.rcount) {
    cudaMemsetAsync(wb.rcount, 0, 4, st);
    refine_select<<<blocks, WAVE_THREADS, 0, st>>>(cp, S, wb, n_pix, out);
    nlaunch++;
    const uint32_t per = std::max(1u, std::min(cp.refine, wave_paths / n_pix));
    for (uint32_t e0 = 0; e0 < cp.refine; e0 += per) {
      const uint32_t n_e = std::min(per, cp.refine - e0);
      cudaMemsetAsync(wb.counts, 0, 16, st);
      WaveBufs w = wb;
      w.q_in = wb.qa; w.count_in = wb.counts + 0;
      refine_gen<<<blocks, WAVE_THREADS, 0, st>>>(*cp2, w, cp.spp, e0, n_e);
      wave_bounces(S, *cp2, wb, WAVE_PLAIN, blocks, st, &nlaunch, timer);
      refine_finalize<<<blocks, WAVE_THREADS, 0, st>>>(cp, wb, cp.spp, e0, n_e, out, e0 + n_e >= cp.refine);
      nlaunch += 2;
    }
  }
  if (launches) *launches += nlaunch;
}

int wave_blocks_per_sm() {
  int a = 0, b = 0, c = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, wave_extend<WAVE_PLAIN, false>, WAVE_THREADS, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, wave_shade<VT_SHADE_PATH, WAVE_PLAIN>, WAVE_THREADS, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, wave_shadow<WAVE_PLAIN, false>, WAVE_THREADS, 0);
  return std::max(1, std::max(a, std::max(b, c)));
}

}  // namespace vtk
