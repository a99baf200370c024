// Differentiable calibration render on sm_103a. The reference has no differentiation (only the analytic dtheta_d /
// dtheta of gpu/lens.js:25); this is the project's own estimator, built from the twin's pieces so that its gradient
// with respect to material albedos and emitter radiances can be computed by path replay.
//
// Estimator (per camera sub-sample, the KB4 ray and sample numbers of the path tracer, gpu/wgsl/kernels.wgsl.js
// :34-53): up to D vertices on Lambertian surfaces (f = rho / pi). At every vertex, nL emitter samples (area CDF,
// power-heuristic MIS against cosine sampling, gpu/wgsl/shade.wgsl.js:135 lightEval); between vertices, cosine-
// weighted continuation, so the throughput gains exactly rho per bounce; at vertex D, the light the node radiosity
// carries: rho / pi x H(node), H = F B the irradiance from the other nodes. An emitter hit adds its radiance
// (MIS-weighted after the first vertex). Nothing in the sampling depends on the parameters, so the estimator is a
// polynomial in the albedos, linear in the emitter radiances and in H, and its derivative is exact by replay:
// each path's record (its vertices' materials and nodes, its light samples' contributions) is differentiated term by
// term, and the derivatives are accumulated in FP64.
//
// The paths are traced by the wavefront kernels of the path tracer (closest hit, then calib_shade, then
// calib_shadow), which write each path's record. When the records of every path fit in memory the backward reads the
// forward's records; otherwise the paths are traced again in chunks of sub-samples, each chunk's records
// differentiated before the next is traced. Both forms trace the same paths with the same kernels, so the replayed
// records are bit-identical to the forward's.
#include <utility>

#include "vt_calib.cuh"
#include "vt_calib_tan.cuh"
#include "vt_camera.cuh"
#include "vt_wave.cuh"

namespace vtk {
using namespace vtd;

namespace {
constexpr int CT = 128;

// append `want` lanes' items to a queue with one atomic per warp; returns the slot of this lane (if want)
__device__ __forceinline__ uint32_t warp_append_c(uint32_t* count, bool want) {
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

struct CalVertex {
  uint32_t mat;
  uint32_t lamp[CAL_MAX_NL];
  float q[CAL_MAX_NL];   // contribution per unit emitter radiance, per unit albedo (0: no contribution)
};
struct CalPath {
  uint32_t n;            // shading vertices
  CalVertex v[CAL_MAX_DEPTH];
  uint32_t emit_lamp;    // emitter hit after the n shading vertices (~0: none)
  float emit_a;          // its MIS weight x profile
  uint32_t node;         // node term at the last shading vertex (~0: none)
};

// the derivative record of a path in d0 (stored form, kept only when the intrinsics' derivative is asked for): each
// light sample's dq (per unit emitter radiance and albedo; cleared with q when the sample is occluded), the emitter
// hit's d a, the ray's tangents between bounces, and the triangle each bounce hit (~0: none)
struct CalTan {
  float dq[CAL_MAX_DEPTH][CAL_MAX_NL][3];
  float de[3];
  Tan3 Jo, Jd;
  float3 dpb;
  uint32_t tri[CAL_MAX_DEPTH], inst[CAL_MAX_DEPTH];
};

// a path's discrete decisions (replay form): per bounce the triangle and instance its extension ray met (~0 and 0xff:
// none), and one bit per vertex and light sample, set when that sample's shadow ray was occluded
struct CalDec {
  uint32_t tri[CAL_MAX_DEPTH];
  uint8_t inst[CAL_MAX_DEPTH];
  uint32_t occ;
};
static_assert(CAL_MAX_DEPTH * CAL_MAX_NL <= 32, "one occlusion bit per vertex and light sample");
static_assert(VT_MAX_INST < 0xff, "instances fit a byte");

// emitter sample by the area CDF, with the index of the triangle (gpu/wgsl/shade.wgsl.js:31)
__device__ __forceinline__ uint32_t sample_emitter_idx(const Scene& S, float3 u, float time, float3& p, float3& n, float3& axis) {
  uint32_t lo = 0, hi = S.emit_n - 1u;
  for (uint32_t it = 0; it < 40u && lo < hi; it++) {
    const uint32_t m = (lo + hi) >> 1;
    if (__ldg(S.params + S.emit_off + 4u * m).w < u.x) lo = m + 1u; else hi = m;
  }
  const float4* e = S.params + S.emit_off + 4u * lo;
  const float3 v0 = xyz(__ldg(e)), e1 = xyz(__ldg(e + 1)), e2 = xyz(__ldg(e + 2)), nl = xyz(__ldg(e + 3));
  const float su = sqrtf(u.y);
  const float3 pl = v0 + e1 * (su * (1.0f - u.z)) + e2 * (su * u.z);
  Rot R;
  float3 pp;
  inst_pose(S, ldu(S.su + 17), time, R, pp);
  p = rmul(R, pl) + pp;
  n = rmul(R, nl);
  axis = rmul(R, ld3(S.su + 4));
  return lo;
}

__device__ __forceinline__ float3 alb(const CalibDev& C, uint32_t m) { return f3(__ldg(C.albedo + 3 * m), __ldg(C.albedo + 3 * m + 1), __ldg(C.albedo + 3 * m + 2)); }

// the emitter hit's weight a = w prof (w = 1 at the first vertex, else pb^2 / (pb^2 + nl^2 pL^2) with
// pL = t^2 / (cosE area)) and its derivative, given the tangents of the ray, of the hit distance and of the
// previous vertex's continuation pdf pb
__device__ __forceinline__ float3 tan_emitter_hit(const Scene& S, const Hit& h, const Surf& s, float3 d, float tt, uint32_t b, float pb, float3 dpb,
                                                 float fnl, float area, const Tan3& Jd, const Tan3& Jx, float3 dt) {
  Tan3 JnE;
  const float3 nE = tan_interp_normal(S, h, s, tt, Jx, JnE);
  const float3 axis = emitter_axis_at(S, tt);
  const float c = clampf(dot(-d, axis), -1.0f, 1.0f);
  const float th = acosf(c);
  const float prof = profile(S, th), slope = profile_slope(S, th);
  const float cosE = dot(-d, nE);
  const float pL = h.t * h.t / (cosE * area);
  const float A = pb * pb, B = fnl * fnl * pL * pL, AB = A + B;
  const float w = b > 1 ? A / AB : 1.0f;
  const float dtv[3] = {dt.x, dt.y, dt.z}, dpbv[3] = {dpb.x, dpb.y, dpb.z};
  float out[3];
  for (int j = 0; j < 3; j++) {
    const float dc = -dot(axis, Jd.c[j]);
    const float dth = (1.0f - c * c) > 0.0f ? -dc / sqrtf(1.0f - c * c) : 0.0f;
    float dw = 0.0f;
    if (b > 1) {
      const float dcosE = -dot(Jd.c[j], nE) - dot(d, JnE.c[j]);
      const float dpL = (2.0f * h.t * dtv[j] * cosE - h.t * h.t * dcosE) / (cosE * cosE * area);
      const float dA = 2.0f * pb * dpbv[j], dB = 2.0f * fnl * fnl * pL * dpL;
      dw = (dA * B - A * dB) / (AB * AB);
    }
    out[j] = dw * prof + w * slope * dth;
  }
  return f3(out[0], out[1], out[2]);
}

// radiance of a recorded path
__device__ __forceinline__ float3 path_value(const CalibDev& C, const CalPath& P, uint32_t nl) {
  float3 L = f3(0, 0, 0), T = f3(1, 1, 1);
  for (uint32_t k = 0; k < P.n; k++) {
    const float3 rho = alb(C, P.v[k].mat);
    float s = 0.0f;
    for (uint32_t j = 0; j < nl; j++) if (P.v[k].q[j] != 0.0f) s += __ldg(C.lamp + P.v[k].lamp[j]) * P.v[k].q[j];
    const float3 Tr = T * rho;
    L = L + Tr * (s / float(nl));
    if (k + 1 == P.n && P.node != MISS) {
      const float3 Hn = f3(__ldg(C.H + P.node), __ldg(C.H + C.n_nodes + P.node), __ldg(C.H + 2 * C.n_nodes + P.node));
      L = L + Tr * Hn * INV_PI_F;
    }
    T = Tr;
  }
  if (P.emit_lamp != MISS) L = L + T * (P.emit_a * __ldg(C.lamp + P.emit_lamp));
  return L;
}

// d loss / d parameters of one recorded path, given g = d loss / d (path radiance); FP64 into shared accumulators
// a path's albedo gradient: per vertex its material and g-weighted value (on: the vertex exists)
struct AlbGrad {
  uint32_t mat[CAL_MAX_DEPTH];
  float3 val[CAL_MAX_DEPTH];
  bool on[CAL_MAX_DEPTH];
};

__device__ __forceinline__ void path_grad(const CalibDev& C, const CalPath& P, uint32_t nl, float3 g, double* sh_lamp, AlbGrad& ag) {
  // Each term is formed in FP32 and added to the FP64 accumulators (FP64 arithmetic runs at a small fraction of
  // this part's FP32 rate; the reductions stay FP64). A term whose albedo product ends at vertex k adds
  // g o value / rho_l to every vertex l <= k: D[k] gathers the g-weighted values of the terms ending at k, and vertex
  // l receives (sum_{k >= l} D[k]) / rho_l, which the caller sums over the warp per material.
  const float fnl = float(nl);
  float3 T = f3(1, 1, 1);
  float3 D[CAL_MAX_DEPTH], rho[CAL_MAX_DEPTH];
#pragma unroll
  for (uint32_t k = 0; k < CAL_MAX_DEPTH; k++) {
    D[k] = f3(0, 0, 0);
    rho[k] = f3(1, 1, 1);
    if (k >= P.n) continue;
    rho[k] = alb(C, P.v[k].mat);
    T = T * rho[k];
    float s = 0.0f;
    for (uint32_t j = 0; j < nl; j++) {
      const float q = P.v[k].q[j];
      if (q == 0.0f) continue;
      atomicAdd(sh_lamp + P.v[k].lamp[j], double(dot(g, T) * q / fnl));
      s += __ldg(C.lamp + P.v[k].lamp[j]) * q;
    }
    if (s != 0.0f) D[k] = D[k] + g * T * (s / fnl);
    if (k + 1 == P.n && P.node != MISS) {
      const float ip = 0.318309886183790672f;
      const float3 Hn = f3(__ldg(C.H + P.node), __ldg(C.H + C.n_nodes + P.node), __ldg(C.H + 2 * C.n_nodes + P.node));
      atomicAdd(C.g_H + P.node, double(g.x * T.x * ip));
      atomicAdd(C.g_H + C.n_nodes + P.node, double(g.y * T.y * ip));
      atomicAdd(C.g_H + 2 * C.n_nodes + P.node, double(g.z * T.z * ip));
      D[k] = D[k] + g * T * Hn * ip;
    }
  }
  if (P.emit_lamp != MISS && P.emit_a != 0.0f) {
    atomicAdd(sh_lamp + P.emit_lamp, double(dot(g, T) * P.emit_a));
    if (P.n) {
      const float Le = P.emit_a * __ldg(C.lamp + P.emit_lamp);
#pragma unroll
      for (uint32_t k = 0; k < CAL_MAX_DEPTH; k++)
        if (k + 1 == P.n) D[k] = D[k] + g * T * Le;
    }
  }
  float3 acc = f3(0, 0, 0);
#pragma unroll
  for (int k = CAL_MAX_DEPTH - 1; k >= 0; k--) {
    ag.on[k] = uint32_t(k) < P.n;
    if (!ag.on[k]) continue;
    acc = acc + D[k];
    ag.mat[k] = P.v[k].mat;
    ag.val[k] = f3(acc.x / rho[k].x, acc.y / rho[k].y, acc.z / rho[k].z);
  }
}

// Adds each lane's value (on: it has one) to sh[3 key + c]: the lanes with the same key are summed over the warp in
// FP32 (a fixed butterfly, so the sum depends only on the warp's lanes), then one FP64 shared atomic per key and
// channel. Called by all 32 lanes of the warp.
__device__ __forceinline__ void warp_key_add3(double* sh, uint32_t key, float3 v, bool on) {
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t pending = __ballot_sync(0xffffffffu, on);
  while (pending) {
    const uint32_t leader = __ffs(pending) - 1;
    const uint32_t k0 = __shfl_sync(0xffffffffu, key, leader);
    const bool in = on && key == k0;
    pending &= ~__ballot_sync(0xffffffffu, in);
    float a = in ? v.x : 0.0f, b = in ? v.y : 0.0f, c = in ? v.z : 0.0f;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
      c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if (lane == leader) {
      atomicAdd(sh + 3 * k0, double(a));
      atomicAdd(sh + 3 * k0 + 1, double(b));
      atomicAdd(sh + 3 * k0 + 2, double(c));
    }
    if (in) on = false;
  }
}

// ------------------------------------------------------------------------------------ the wavefront estimator
// The estimator split like the path tracer: the closest-hit kernel of the wavefront, then calib_shade (one vertex:
// the record of the vertex, its light samples' unshadowed contributions and shadow segments, the cosine
// continuation), then calib_shadow (any hit per light sample; an occluded sample's contribution is cleared in the
// record). Each path's record (CalPath) stays in HBM, so the backward evaluates path_grad on the records without
// tracing again. Records of path (i, id) of a camera's sub-samples [i0, i1) sit at rec[(i - i0) n_pix + id].
constexpr int WT = 256;

template <bool TAN>
__global__ void __launch_bounds__(WT, 3) calib_shade_kernel(const Scene S, const CamParams cp, const CalibDev C, WaveBufs wb, CalPath* rec,
                                                        CalTan* tan, uint32_t b, CalDec* dec, int dmode) {
  const uint32_t n = *wb.count_in;
  const uint32_t nl = cp.n_light;
  const float fnl = float(nl);
  const float area = __ldg(S.su + 3);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const uint32_t p = wb.q_in[k];
    CalPath& P = rec[p];
    if (b == 1) { P.n = 0; P.emit_lamp = MISS; P.emit_a = 0.0f; P.node = MISS; }
    const uint4 meta = wb.meta[p];
    const uint32_t i = meta.y, hs = meta.z;
    const float4 o4 = wb.o[p], d4 = wb.d[p], hv = wb.hit[p];
    const float3 o = xyz(o4), d = xyz(d4);
    const float tt = o4.w, pb_prev = d4.w;
    const Hit h{hv.x, hv.y, hv.z, __float_as_uint(hv.w), wb.hinst[p]};
    if (dmode == 1) {
      CalDec& D = dec[p];
      // every bounce of the path starts as none: a replay whose path continues where the recorded one stopped (its
      // rays can differ from the recorded ones in the last bits) meets nothing there, never a stale triangle
      if (b == 1) {
        D.occ = 0u;
        for (uint32_t a = 0; a < CAL_MAX_DEPTH; a++) { D.tri[a] = MISS; D.inst[a] = uint8_t(0xff); }
      }
      D.tri[b - 1] = h.tri;
      D.inst[b - 1] = h.inst == MISS ? uint8_t(0xff) : uint8_t(h.inst);
    }
    const uint32_t occ = dmode == 2 ? dec[p].occ : 0u;
    bool cont = false, shadow = false;
    Tan3 Jo, Jd, Jx;
    float3 dpb, dt;
    if (TAN) {
      CalTan& G = tan[p];
      if (b == 1) {
        for (uint32_t a = 0; a < CAL_MAX_DEPTH; a++) {
          G.tri[a] = MISS; G.inst[a] = MISS;
          for (uint32_t j = 0; j < CAL_MAX_NL; j++) G.dq[a][j][0] = G.dq[a][j][1] = G.dq[a][j][2] = 0.0f;
        }
        G.de[0] = G.de[1] = G.de[2] = 0.0f;
        Jo = tan_zero(); Jd = tan_identity(); dpb = f3(0, 0, 0);
      } else {
        Jo = G.Jo; Jd = G.Jd; dpb = G.dpb;
      }
      G.tri[b - 1] = h.tri;
      G.inst[b - 1] = h.inst;
    }
    if (h.tri != MISS) {
      const Surf s = surface(S, h, o, d, tt);
      if (TAN) tan_plane_hit(Jo, Jd, d, s.ng, h.t, Jx, dt);
      if (s.flags & VT_F_EMITTER) {
        const float3 nE = emitter_normal(S, h, s, tt);
        const float cosE = dot(-d, nE);
        if (cosE > 0.0f) {
          const float prof = profile(S, acosf(clampf(dot(-d, emitter_axis_at(S, tt)), -1.0f, 1.0f)));
          float w = 1.0f;
          if (b > 1) {
            const float pL = h.t * h.t / (cosE * area);
            w = pb_prev * pb_prev / (pb_prev * pb_prev + fnl * fnl * pL * pL);
          }
          P.emit_lamp = __ldg(C.emit_of_tri + h.tri);
          P.emit_a = w * prof;
          if (TAN) {
            const float3 de = tan_emitter_hit(S, h, s, d, tt, b, pb_prev, dpb, fnl, area, Jd, Jx, dt);
            tan[p].de[0] = de.x; tan[p].de[1] = de.y; tan[p].de[2] = de.z;
          }
        }
      } else {
        const uint32_t vk = P.n;
        CalVertex& V = P.v[vk];
        V.mat = s.mat;
        P.n = vk + 1;
        const float3 nrm = s.ns, wo = -d;
        Tan3 Jn;
        if (TAN) Jn = tan_shading_normal(S, h, s, tt, Jx);
        const float sh0 = b == 1 ? u01(pcg(hs + 3u)) : bounce_shift(hs, b, 0);
        const float sh1 = b == 1 ? u01(pcg(hs + 4u)) : bounce_shift(hs, b, 1);
        const float sh2 = b == 1 ? u01(pcg(hs + 5u)) : bounce_shift(hs, b, 2);
        float4* srec = wb.sh + size_t(p) * nl * 3;
        for (uint32_t j = 0; j < nl; j++) {
          const float3 u = f3(kr(i * nl + j, KL0, sh0), kr(i * nl + j, KL1, sh1), kr(i * nl + j, KL2, sh2));
          float3 lp, ln, la;
          V.lamp[j] = sample_emitter_idx(S, u, tt, lp, ln, la);
          V.q[j] = 0.0f;
          srec[3 * j + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          float3 wi = lp - s.p;
          const float d2 = dot(wi, wi), dist = sqrtf(d2);
          wi = wi / dist;
          const float cosE = dot(-wi, ln), cosS = dot(nrm, wi);
          if (cosE <= 0.0f || cosS <= 0.0f || dot(s.ng, wi) <= 0.0f || dot(nrm, wo) <= 0.0f) continue;
          const float prof = profile(S, acosf(clampf(dot(-wi, la), -1.0f, 1.0f)));
          if (prof <= 0.0f) continue;
          const float pdfW = d2 / (cosE * area), pb = cosS * INV_PI_F;
          const float w = fnl * fnl * pdfW * pdfW / (fnl * fnl * pdfW * pdfW + pb * pb);
          V.q[j] = prof * cosS * w * INV_PI_F / pdfW;
          if (TAN) {
            const float3 dq = tan_light(S, s.p, nrm, lp, ln, la, area, fnl, V.q[j], Jx, Jn);
            tan[p].dq[vk][j][0] = dq.x; tan[p].dq[vk][j][1] = dq.y; tan[p].dq[vk][j][2] = dq.z;
          }
          if (dmode == 2) {
            // the recorded shadow ray's outcome: an occluded sample is cleared as calib_shadow_kernel clears it
            if ((occ >> (vk * CAL_MAX_NL + j)) & 1u) {
              V.q[j] = 0.0f;
              if (TAN) tan[p].dq[vk][j][0] = tan[p].dq[vk][j][1] = tan[p].dq[vk][j][2] = 0.0f;
            }
            continue;
          }
          const float3 so = offset_ray(s.p, s.ng, wi);
          srec[3 * j] = make_float4(so.x, so.y, so.z, dist - 2e-5f);
          srec[3 * j + 1] = make_float4(wi.x, wi.y, wi.z, 1.0f);
          srec[3 * j + 2] = make_float4(0.0f, 0.0f, __uint_as_float(vk), 0.0f);
          shadow = true;
        }
        if (shadow) wb.nee[p] = make_float4(0.0f, 0.0f, 0.0f, tt);
        if (b == cp.max_depth) {
          if (h.inst == MISS && h.tri < C.n_static_tris) P.node = __ldg(C.tri_node + h.tri);
        } else if (dot(nrm, wo) > 0.0f) {
          const float u1 = b == 1 ? kr(i, KB1, u01(pcg(hs + 7u))) : kr(i, KB1, bounce_shift(hs, b, 4));
          const float u2 = b == 1 ? kr(i, KB2, u01(pcg(hs + 8u))) : kr(i, KB2, bounce_shift(hs, b, 5));
          const float3 t = basis_t(nrm), bb = basis_b(nrm);
          const float r = sqrtf(u1);
          float sp, cpz;
          sincosf(2.0f * PI_F * u2, &sp, &cpz);
          const float3 l = t * (r * cpz) + bb * (r * sp) + nrm * sqrtf(fmaxf(0.0f, 1.0f - u1));
          const float cl = dot(nrm, l);
          if (cl > 0.0f && dot(s.ng, l) > 0.0f) {
            const float3 no = offset_ray(s.p, s.ng, l);
            wb.o[p] = make_float4(no.x, no.y, no.z, tt);
            wb.d[p] = make_float4(l.x, l.y, l.z, cl * INV_PI_F);
            wb.meta[p] = make_uint4(meta.x, meta.y, meta.z, b + 1u);
            cont = true;
            if (TAN) {
              const Tan3 Jl = tan_continue(nrm, Jn, r, cpz, sp, sqrtf(fmaxf(0.0f, 1.0f - u1)));
              tan[p].dpb = (tan_dot(l, Jn) + tan_dot(nrm, Jl)) * INV_PI_F;
              tan[p].Jo = Jx;
              tan[p].Jd = Jl;
            }
          }
        }
      }
    }
    const uint32_t qs = warp_append_c(wb.count_out, cont);
    if (cont) wb.q_out[qs] = p;
    const uint32_t ss = warp_append_c(wb.count_sh, shadow);
    if (shadow) wb.q_sh[ss] = p;
  }
}

// any hit of the pending light samples on persistent lanes; an occluded sample's contribution is cleared in the record
template <bool TAN>
__global__ void __launch_bounds__(WT, 4) calib_shadow_kernel(const Scene S, const CamParams cp, WaveBufs wb, CalPath* rec, CalTan* tan, CalDec* dec) {
  const uint32_t n = *wb.count_sh;
  const uint32_t nl = cp.n_light;
  const uint32_t skip = ldu(S.su + 7);
  __shared__ uint2 stack_sh[SH_DEPTH * WT];
  LaneStack stk;
  stk.sh = stack_sh; stk.lane = threadIdx.x; stk.stride = WT;
  TraceState st;
  float3 o = f3(0, 0, 0), d = f3(0, 0, 1);
  float tt = 0.0f;
  uint32_t p = 0, j = 0;
  bool active = false, exhausted = false;
  const float4* srec = nullptr;
  auto next_sample = [&]() -> bool {
    for (; j < nl; j++) {
      const float4 a = srec[3 * j], w = srec[3 * j + 1];
      if (w.w == 0.0f) continue;
      o = xyz(a); d = xyz(w);
      st.best = Hit{a.w, 0.0f, 0.0f, MISS, MISS};
      if (trace_phase(S, cp.root, o, d, 0.0f, tt, 3u, skip, st, -1)) return true;
    }
    return false;
  };
  auto start = [&](uint32_t idx) {
    p = wb.q_sh[idx];
    tt = wb.nee[p].w;
    srec = wb.sh + size_t(p) * nl * 3;
    j = 0;
    active = next_sample();
  };
  while (take_rays(active, exhausted, wb.fetch, n, cp.refill, start)) {
    if (!active) continue;
    const int r = trace_step<true>(S, 0.0f, st, stk);
    bool done = r == 2;
    if (r == 1) done = !trace_phase(S, cp.root, o, d, 0.0f, tt, 3u, skip, st, st.k + 1);
    if (!done) continue;
    if (st.best.tri != MISS) {
      const uint32_t vk = __float_as_uint(srec[3 * j + 2].z);
      rec[p].v[vk].q[j] = 0.0f;
      if (TAN) tan[p].dq[vk][j][0] = tan[p].dq[vk][j][1] = tan[p].dq[vk][j][2] = 0.0f;
      if (dec) dec[p].occ |= 1u << (vk * CAL_MAX_NL + j);
    }
    j++;
    active = next_sample();
  }
}

// per pixel: the image value from the records in sub-sample order, its loss partial (forward); or the gradient of
// every record (backward)
// the derivative in d0 of a recorded path's radiance, per channel, from its derivative record
__device__ __forceinline__ void path_tangent(const CalibDev& C, const CalPath& P, const CalTan& G, uint32_t nl, float3* dL) {
  dL[0] = dL[1] = dL[2] = f3(0, 0, 0);
  float3 T = f3(1, 1, 1);
  for (uint32_t k = 0; k < P.n; k++) {
    T = mul3(T, alb(C, P.v[k].mat));
    for (uint32_t j = 0; j < nl; j++) {
      if (P.v[k].q[j] == 0.0f) continue;
      const float3 dq = f3(G.dq[k][j][0], G.dq[k][j][1], G.dq[k][j][2]) * (__ldg(C.lamp + P.v[k].lamp[j]) / float(nl));
      dL[0] = dL[0] + dq * T.x; dL[1] = dL[1] + dq * T.y; dL[2] = dL[2] + dq * T.z;
    }
  }
  if (P.emit_lamp != MISS) {
    const float3 de = f3(G.de[0], G.de[1], G.de[2]) * __ldg(C.lamp + P.emit_lamp);
    dL[0] = dL[0] + de * T.x; dL[1] = dL[1] + de * T.y; dL[2] = dL[2] + de * T.z;
  }
}

// the derivative of the loss in the camera's intrinsics from one sub-sample: G = g . dL / d d0 (FP64), chained
// through d d0 / d K at the sub-sample's image position
__device__ __forceinline__ void add_intrinsics_grad(const CamParams& cp, uint32_t id, uint32_t i, const float3* dL, double3 g, float* kacc) {
  uint32_t x, y;
  if (!pixel_xy(cp, id, x, y)) return;
  // the term in FP32, its accumulation in FP64
  const float gx = float(g.x), gy = float(g.y), gz = float(g.z);
  const float G[3] = {gx * dL[0].x + gy * dL[1].x + gz * dL[2].x, gx * dL[0].y + gy * dL[1].y + gz * dL[2].y,
                      gx * dL[0].z + gy * dL[1].z + gz * dL[2].z};
  if (G[0] == 0.0f && G[1] == 0.0f && G[2] == 0.0f) return;
  const uint32_t hs = hash3(x, y, cp.seed * 64u + cp.cam_index);
  const float2 uv = subsample_uv(x, y, i, hs);
  float J[3][8];
  kb4_ray_jacobian(cp.lens, uv.x, uv.y, f3(cp.rx[0], cp.rx[1], cp.rx[2]), f3(cp.ry[0], cp.ry[1], cp.ry[2]), f3(cp.rz[0], cp.rz[1], cp.rz[2]), J);
#pragma unroll
  for (int k = 0; k < 8; k++) kacc[k] += G[0] * J[0][k] + G[1] * J[1][k] + G[2] * J[2][k];
}

// per pixel over the records of sub-samples [i0, i1): backward 0 adds their values to the pixel's running sum (kept in
// the image between chunks; the chunk that ends at spp writes the image and the loss partials), 1 / 2 accumulate the
// gradients (2: with the intrinsics' derivative)
__global__ void __launch_bounds__(CT) calib_records_kernel(const CamParams cp, const CalibDev C, const CalPath* __restrict__ rec,
                                                          const CalTan* __restrict__ tan, uint32_t n_pix, int backward, uint32_t i0,
                                                          uint32_t i1) {
  extern __shared__ double sm[];
  double* sh_alb = sm;
  double* sh_lamp = sm + 3 * C.n_mat;
  __shared__ double red[CT / 32];
  __shared__ double sh_k[8];
  if (backward) {
    for (uint32_t k = threadIdx.x; k < 3 * C.n_mat + C.n_lamps; k += blockDim.x) sm[k] = 0.0;
    if (threadIdx.x < 8) sh_k[threadIdx.x] = 0.0;
    __syncthreads();
  }
  double loss = 0.0;
  // the thread's intrinsics terms (one pixel's sub-samples of the launch) summed in FP32 registers, then one FP64 warp
  // sum and 8 shared atomics per warp at the end: all lanes add to the same 8 words, where per-path atomics would
  // contend, and FP64 issues at a small fraction of FP32 on this part
  float kacc[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  const float sc = cp.scale / float(cp.spp);
  // the block's threads take pixels base + threadIdx.x together, so that a warp's lanes stay together for the
  // per-material warp sums of the backward
  for (uint32_t base = blockIdx.x * blockDim.x; base < n_pix; base += gridDim.x * blockDim.x) {
    const uint32_t id = base + threadIdx.x;
    uint32_t x = 0, y = 0;
    const bool valid = id < n_pix && pixel_xy(cp, id, x, y);
    const size_t px = size_t(y) * cp.w + x;
    if (backward) {
      double3 g = make_double3(0.0, 0.0, 0.0);
      if (valid) {
        const float4 I = C.image[px], Tg = C.target ? C.target[px] : make_float4(0.f, 0.f, 0.f, 0.f);
        const double k = 2.0 * C.inv_count * double(sc);
        g = make_double3(k * (double(I.x) - Tg.x), k * (double(I.y) - Tg.y), k * (double(I.z) - Tg.z));
      }
      const float3 gf = f3(float(g.x), float(g.y), float(g.z));
      for (uint32_t i = i0; i < i1; i++) {
        const size_t r = size_t(i - i0) * n_pix + id;
        AlbGrad ag;
#pragma unroll
        for (uint32_t k = 0; k < CAL_MAX_DEPTH; k++) { ag.on[k] = false; ag.mat[k] = 0u; ag.val[k] = f3(0, 0, 0); }
        if (valid) path_grad(C, rec[r], cp.n_light, gf, sh_lamp, ag);
#pragma unroll
        for (uint32_t k = 0; k < CAL_MAX_DEPTH; k++) warp_key_add3(sh_alb, ag.mat[k], ag.val[k], ag.on[k]);
        if (backward == 2 && valid) {
          float3 dL[3];
          path_tangent(C, rec[r], tan[r], cp.n_light, dL);
          add_intrinsics_grad(cp, id, i, dL, g, kacc);
        }
      }
    } else {
      if (!valid) continue;
      // the sum over sub-samples in order, carried across chunks exactly (a float in the image)
      float3 s = f3(0, 0, 0);
      if (i0 > 0) s = xyz(C.image[px]);
      for (uint32_t i = i0; i < i1; i++) s = s + path_value(C, rec[size_t(i - i0) * n_pix + id], cp.n_light);
      if (i1 < cp.spp) {
        C.image[px] = make_float4(s.x, s.y, s.z, 0.0f);
        continue;
      }
      const float4 I = make_float4(s.x * sc, s.y * sc, s.z * sc, 1.0f);
      C.image[px] = I;
      if (C.target) {
        const float4 Tg = C.target[px];
        const double dx = double(I.x) - Tg.x, dy = double(I.y) - Tg.y, dz = double(I.z) - Tg.z;
        loss += dx * dx + dy * dy + dz * dz;
      }
    }
  }
  if (backward) {
    if (backward == 2) {
#pragma unroll
      for (int k = 0; k < 8; k++) {
        double v = double(kacc[k]);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31u) == 0u && v != 0.0) atomicAdd(sh_k + k, v);
      }
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < 3 * C.n_mat; k += blockDim.x) if (sm[k] != 0.0) atomicAdd(C.g_albedo + k, sm[k]);
    for (uint32_t k = threadIdx.x; k < C.n_lamps; k += blockDim.x) if (sh_lamp[k] != 0.0) atomicAdd(C.g_lamp + k, sh_lamp[k]);
    if (backward == 2 && threadIdx.x < 8 && sh_k[threadIdx.x] != 0.0) atomicAdd(C.g_K + threadIdx.x, sh_k[threadIdx.x]);
    return;
  }
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = loss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < CT / 32; w++) t += red[w];
    C.partials[blockIdx.x] = t * C.inv_count;
  }
}

// one thread per (node, emitter triangle): stratified points (Kronecker in the unit square, the sampler's
// triangle warp), cosines, profile, visibility through the BVH
__global__ void direct_transfer_kernel(const Scene S, const float* __restrict__ C, const float* __restrict__ N, uint32_t n, uint32_t n_lamps,
                                       uint32_t samples, float* __restrict__ D) {
  const size_t total = size_t(n) * n_lamps;
  const uint32_t skip = ldu(S.su + 7);
  for (size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x; k < total; k += size_t(gridDim.x) * blockDim.x) {
    const uint32_t i = uint32_t(k / n_lamps), t = uint32_t(k % n_lamps);
    const float3 c = f3(C[3 * i], C[3 * i + 1], C[3 * i + 2]), nn = f3(N[3 * i], N[3 * i + 1], N[3 * i + 2]);
    const float4* e = S.params + S.emit_off + 4u * t;
    const float3 v0 = xyz(__ldg(e)), e1 = xyz(__ldg(e + 1)), e2 = xyz(__ldg(e + 2)), nl0 = xyz(__ldg(e + 3));
    const float At = 0.5f * length(cross(e1, e2));
    Rot R;
    float3 pp;
    inst_pose(S, ldu(S.su + 17), 0.5f, R, pp);
    const float3 nl = rmul(R, nl0), axis = rmul(R, ld3(S.su + 4));
    const float3 org = c + nn * 1e-4f;
    float acc = 0.0f;
    for (uint32_t s = 0; s < samples; s++) {
      const float u1 = kr(s, R2A, 0.5f), u2 = kr(s, R2B, 0.5f);
      const float su = sqrtf(u1);
      const float3 lp = rmul(R, v0 + e1 * (su * (1.0f - u2)) + e2 * (su * u2)) + pp;
      float3 w = lp - org;
      const float r2 = dot(w, w), r = sqrtf(r2);
      w = w / r;
      const float ci = dot(nn, w), ct = dot(nl, -w);
      if (ci <= 0.0f || ct <= 0.0f) continue;
      const float prof = profile(S, acosf(clampf(dot(-w, axis), -1.0f, 1.0f)));
      if (prof <= 0.0f) continue;
      const Hit h = trace_scene<true>(S, 0u, org, w, 0.0f, r - 2e-5f, 0.5f, 3u, skip);
      if (h.tri == MISS) acc += prof * ci * ct / r2;
    }
    D[size_t(i) * n_lamps + t] = acc * At / float(samples);
  }
}

__global__ void dl_kernel(const float* __restrict__ D, const float* __restrict__ L, uint32_t n, uint32_t n_lamps, float* __restrict__ y) {
  const uint32_t row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
  if (row >= n) return;
  float a = 0.0f;
  for (uint32_t t = lane; t < n_lamps; t += 32) a = fmaf(D[size_t(row) * n_lamps + t], L[t], a);
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) y[row] = a;
}

// The calibration's node radiosity and its adjoint at FP64 accuracy without FP64 inner products (FP64 issues at a
// small fraction of FP32 on this part): a vector entry x is held as the float pair (hi, lo) with hi = float(x),
// lo = float(x - hi); each product F_ij x_j is formed exactly for hi by an FMA (its rounding error) plus the lo
// part's product, and the products are summed in a float pair by compensated addition (two-sum, then renormalised).
// Each step is good to about 2^-48 relative; a float32 restatement of 4096-term sums measures at most about 1e-13
// relative against exact sums (FP32 alone: 1e-6). Rows, columns and splits meet in FP64.
__device__ __forceinline__ float2 df_split(double x) {
  const float h = float(x);
  return make_float2(h, float(x - double(h)));
}
// each step rounded on its own (the _rn intrinsics are never contracted into a multiply-add)
__device__ __forceinline__ void df_mac(float f, float2 x, float& sh, float& sl) {
  const float p = __fmul_rn(f, x.x);
  const float e = __fmaf_rn(f, x.y, __fmaf_rn(f, x.x, -p));
  const float t = __fadd_rn(sh, p);
  const float v = __fsub_rn(t, sh);
  const float lo = __fadd_rn(sl, __fadd_rn(__fadd_rn(__fsub_rn(sh, __fsub_rn(t, v)), __fsub_rn(p, v)), e));
  sh = __fadd_rn(t, lo);                    // renormalised, so that lo stays below an ulp of the sum
  sl = __fsub_rn(lo, __fsub_rn(sh, t));
}

// 64 row splits, so that a sweep has blocks enough to fill the SMs several times (16 splits took 2.7x as long under
// ncu); a thread sums its column's rows in two interleaved float pairs (two independent dependency chains), which
// meet in FP64
constexpr uint32_t JT_SPLITS = 64, JT_COLS = 256;
// partial[split][j] = sum over rows i of the split of F[i][j] (g_i + rho_i lam_i)
__global__ void __launch_bounds__(JT_COLS) jacobi_t_kernel(const float* __restrict__ F, const double* __restrict__ g, const float* __restrict__ rho,
                                                          const double* __restrict__ lam, uint32_t n, double* __restrict__ part) {
  __shared__ float2 w[JT_COLS];
  const uint32_t j = blockIdx.x * JT_COLS + threadIdx.x;
  const uint32_t rows = (n + JT_SPLITS - 1) / JT_SPLITS, i0 = blockIdx.y * rows, i1 = min(n, i0 + rows);
  float sh0 = 0.0f, sl0 = 0.0f, sh1 = 0.0f, sl1 = 0.0f;
  for (uint32_t ib = i0; ib < i1; ib += JT_COLS) {
    const uint32_t ii = ib + threadIdx.x;
    w[threadIdx.x] = ii < i1 ? df_split(g[ii] + double(rho[ii]) * lam[ii]) : make_float2(0.0f, 0.0f);
    __syncthreads();
    const uint32_t m = min(JT_COLS, i1 - ib);
    if (j < n) {
      const float* Fc = F + size_t(ib) * n + j;
      uint32_t k = 0;
      for (; k + 1 < m; k += 2) {
        const float f0 = Fc[size_t(k) * n], f1 = Fc[size_t(k + 1) * n];
        df_mac(f0, w[k], sh0, sl0);
        df_mac(f1, w[k + 1], sh1, sl1);
      }
      if (k < m) df_mac(Fc[size_t(k) * n], w[k], sh0, sl0);
    }
    __syncthreads();
  }
  if (j < n) part[size_t(blockIdx.y) * n + j] = (double(sh0) + double(sl0)) + (double(sh1) + double(sl1));
}
__global__ void jacobi_t_combine(const double* __restrict__ part, uint32_t n, double* __restrict__ out) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double a = 0.0;
  for (uint32_t s = 0; s < JT_SPLITS; s++) a += part[size_t(s) * n + j];
  out[j] = a;
}

// The three channels' B_c,out = rho_c o (DL + F B_c,in) at FP64 accuracy (F in FP32, B as float pairs planar [c][n],
// the products summed in float pairs), one warp per row reading F once for all three; with `H` set, H_c = F B_c,in
// (rounded to FP32) instead. Each channel's sums run in the order of a one-channel sweep, so the values are its.
__global__ void __launch_bounds__(256) radiosity64_kernel(const float* __restrict__ F, const float* __restrict__ rho, const float* __restrict__ DL,
                                                        const float2* __restrict__ Bin, float2* __restrict__ Bout, float* __restrict__ H,
                                                        uint32_t n) {
  const uint32_t row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
  if (row >= n) return;
  const float* Fr = F + size_t(row) * n;
  float sh[3] = {0.0f, 0.0f, 0.0f}, sl[3] = {0.0f, 0.0f, 0.0f};
  if ((n & 3u) == 0u && ((reinterpret_cast<uintptr_t>(F) | reinterpret_cast<uintptr_t>(Bin)) & 15u) == 0u) {
    const float4* F4 = reinterpret_cast<const float4*>(Fr);
    for (uint32_t j = lane; j < (n >> 2); j += 32) {
      const float4 f = __ldg(F4 + j);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const float4* B4 = reinterpret_cast<const float4*>(Bin + size_t(c) * n);   // two pairs per float4
        const float4 b01 = __ldg(B4 + 2 * j), b23 = __ldg(B4 + 2 * j + 1);
        df_mac(f.x, make_float2(b01.x, b01.y), sh[c], sl[c]);
        df_mac(f.y, make_float2(b01.z, b01.w), sh[c], sl[c]);
        df_mac(f.z, make_float2(b23.x, b23.y), sh[c], sl[c]);
        df_mac(f.w, make_float2(b23.z, b23.w), sh[c], sl[c]);
      }
    }
  } else {
    for (uint32_t j = lane; j < n; j += 32) {
      const float f = __ldg(Fr + j);
#pragma unroll
      for (int c = 0; c < 3; c++) df_mac(f, Bin[size_t(c) * n + j], sh[c], sl[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double a = double(sh[c]) + double(sl[c]);
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane) continue;
    if (H) H[size_t(c) * n + row] = float(a);
    else Bout[size_t(c) * n + row] = df_split(double(rho[size_t(c) * n + row]) * (double(DL[row]) + a));
  }
}
__global__ void radiosity64_init(const float* __restrict__ rho, const float* __restrict__ DL, float2* __restrict__ B, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 3 * n) B[i] = df_split(double(rho[i]) * double(DL[i % n]));
}

__global__ void mul_kernel(const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ y, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a[i] * b[i];
}

__global__ void sum_kernel(const double* __restrict__ p, uint32_t n, double* __restrict__ out) {
  __shared__ double s[1024];
  double a = 0.0;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) a += p[i];
  s[threadIdx.x] = a;
  __syncthreads();
  for (uint32_t o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}
// calib_shade_kernel's grid-stride loop runs as one wave of its own occupancy (3 blocks of 256 per SM at 80
// registers) rather than on the traversal kernels' grid, a wave and a third of it (C4 forward 200 -> 196 ms)
template <bool TAN>
int calib_shade_grid() {
  static std::atomic<int> grid[MAX_DEVICES];
  return per_device_value(grid, [](int dev) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, calib_shade_kernel<TAN>, WT, 0);
    return device_sms(dev) * std::max(1, per);
  });
}
}  // namespace

size_t calib_record_bytes(uint32_t paths) { return size_t(paths) * sizeof(CalPath); }

size_t calib_tan_bytes(uint32_t paths) { return size_t(paths) * sizeof(CalTan); }

// the paths of sub-samples [i0, i1) of the camera through the wavefront, their records at rec[(i - i0) n_pix + id]
// tri_hit's arithmetic without its range checks: for a hit tri_hit accepted, the same t, u, v; a recorded hit is met
// again even when the ray moved by rounding (the derivative-record kernel's ray can differ from the plain kernel's
// in its last bits)
__device__ __forceinline__ void tri_uvt(const Scene& S, uint32_t k, float3 o, float3 d, float& t, float& u, float& v) {
  const float4* r = S.tris + 4u * k;
  const float3 v0 = xyz(__ldg(r)), e1 = xyz(__ldg(r + 1)), e2 = xyz(__ldg(r + 2));
  const float3 p = cross(d, e2);
  const float det = dot(e1, p);
  const float inv = 1.0f / det;
  const float3 s = o - v0;
  u = dot(s, p) * inv;
  const float3 q = cross(s, e1);
  v = dot(d, q) * inv;
  t = dot(e2, q) * inv;
}

// the extension rays of a replayed bounce meet the triangles the traced bounce recorded: the traversal's frame (the
// world, or the instance's pose at the path's time) and its triangle arithmetic, so t, u, v are the traced hit's
__global__ void __launch_bounds__(256) calib_rehit_kernel(const Scene S, WaveBufs wb, const CalDec* __restrict__ dec, uint32_t b) {
  const uint32_t n = *wb.count_in;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const uint32_t p = wb.q_in[k];
    const uint32_t tri = dec[p].tri[b - 1], inst = dec[p].inst[b - 1];
    float4 hit = make_float4(BIG, 0.0f, 0.0f, __uint_as_float(MISS));
    uint32_t hinst = MISS;
    if (tri != MISS) {
      const float4 o4 = wb.o[p], d4 = wb.d[p];
      float3 o = xyz(o4), d = xyz(d4);
      if (inst != 0xffu) {
        Rot R;
        float3 pp;
        inst_pose(S, inst, o4.w, R, pp);
        o = rtmul(R, o - pp);
        d = rtmul(R, d);
        hinst = inst;
      }
      float t, u, v;
      tri_uvt(S, tri, o, d, t, u, v);
      hit = make_float4(t, u, v, __uint_as_float(tri));
    }
    wb.hit[p] = hit;
    wb.hinst[p] = hinst;
  }
}

static void calib_trace(const Scene& S, const CamParams& cp, const CalibDev& C, WaveBufs wb, uint32_t wave_paths, CalPath* rec, CalTan* tan,
                        uint32_t i0, uint32_t i1, int blocks, cudaStream_t st, CalDec* dec, int dmode) {
  const uint32_t n_pix = tiled_pixels(cp.w, cp.h, cp.tile_w, cp.tile_h);
  const uint32_t per_wave = std::max(1u, std::min(i1 - i0, wave_paths / std::max(1u, n_pix)));
  for (uint32_t w0 = i0; w0 < i1; w0 += per_wave) {
    const uint32_t n_i = std::min(per_wave, i1 - w0);
    cudaMemsetAsync(wb.counts, 0, 16, st);
    launch_wave_gen(cp, wb, w0, n_i, n_pix, blocks, st);
    CalPath* rb = rec + size_t(w0 - i0) * n_pix;
    CalTan* tb = tan ? tan + size_t(w0 - i0) * n_pix : nullptr;
    CalDec* db = dec && dmode ? dec + size_t(w0) * n_pix : nullptr;
    const int dm = db ? dmode : 0;
    for (uint32_t b = 1; b <= cp.max_depth; b++) {
      WaveBufs w = wb;
      w.q_in = (b & 1) ? wb.qa : wb.qb;
      w.q_out = (b & 1) ? wb.qb : wb.qa;
      w.count_in = wb.counts + ((b & 1) ? 0 : 1);
      w.count_out = wb.counts + ((b & 1) ? 1 : 0);
      w.count_sh = wb.counts + 2;
      cudaMemsetAsync(w.count_out, 0, 4, st);
      cudaMemsetAsync(w.count_sh, 0, 4, st);
      if (dm == 2) calib_rehit_kernel<<<std::max(1, blocks), 256, 0, st>>>(S, w, db, b);
      else launch_wave_extend(S, cp, w, blocks, st);
      if (tb) calib_shade_kernel<true><<<calib_shade_grid<true>(), WT, 0, st>>>(S, cp, C, w, rb, tb, b, db, dm);
      else calib_shade_kernel<false><<<calib_shade_grid<false>(), WT, 0, st>>>(S, cp, C, w, rb, nullptr, b, db, dm);
      if (dm == 2) continue;   // the recorded shadow outcomes were applied by the shading
      cudaMemsetAsync(w.fetch, 0, 4, st);
      if (tb) calib_shadow_kernel<true><<<blocks, WT, 0, st>>>(S, cp, w, rb, tb, db);
      else calib_shadow_kernel<false><<<blocks, WT, 0, st>>>(S, cp, w, rb, nullptr, db);
    }
  }
}

uint32_t calib_wave_forward(const Scene& S, const CamParams& cp, const CalibDev& C, WaveBufs wb, uint32_t wave_paths, void* records, void* tangents,
                            int blocks, cudaStream_t st) {
  return calib_wave_chunk(S, cp, C, wb, wave_paths, records, tangents, 0, cp.spp, 0, blocks, st);
}

size_t calib_dec_bytes(uint32_t paths) { return size_t(paths) * sizeof(CalDec); }

uint32_t calib_wave_chunk(const Scene& S, const CamParams& cp, const CalibDev& C, WaveBufs wb, uint32_t wave_paths, void* records, void* tangents,
                          uint32_t i0, uint32_t i1, int mode, int blocks, cudaStream_t st, void* decisions, int dec_mode) {
  CalPath* rec = static_cast<CalPath*>(records);
  CalTan* tan = static_cast<CalTan*>(tangents);
  calib_trace(S, cp, C, wb, wave_paths, rec, tan, i0, i1, blocks, st, static_cast<CalDec*>(decisions), dec_mode);
  const uint32_t n_pix = tiled_pixels(cp.w, cp.h, cp.tile_w, cp.tile_h);
  const uint32_t grid = std::max(1u, std::min(uint32_t(blocks), (n_pix + CT - 1) / CT));
  const size_t smem = mode ? size_t(3 * C.n_mat + C.n_lamps) * 8 : 0;
  calib_records_kernel<<<grid, CT, smem, st>>>(cp, C, rec, tan, n_pix, mode, i0, i1);
  return grid;
}

void calib_records_backward(const CamParams& cp, const CalibDev& C, const void* records, const void* tangents, int blocks, cudaStream_t st) {
  const uint32_t n_pix = tiled_pixels(cp.w, cp.h, cp.tile_w, cp.tile_h);
  const uint32_t grid = std::max(1u, std::min(uint32_t(blocks), (n_pix + CT - 1) / CT));
  calib_records_kernel<<<grid, CT, size_t(3 * C.n_mat + C.n_lamps) * 8, st>>>(cp, C, static_cast<const CalPath*>(records),
                                                                             static_cast<const CalTan*>(tangents), n_pix, tangents ? 2 : 1,
                                                                             0, cp.spp);
}

// per path of the camera's records, in (row, column, sub-sample) order: the triangle and instance of each bounce
// (~0: none) and each vertex's light samples' q (0: occluded or no contribution)
__global__ void calib_export_paths_kernel(const CamParams cp, const CalPath* __restrict__ rec, const CalTan* __restrict__ tan, uint32_t n_pix,
                                          uint32_t* __restrict__ tri_inst, float* __restrict__ q) {
  const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t x, y;
  if (id >= n_pix || !pixel_xy(cp, id, x, y)) return;
  for (uint32_t i = 0; i < cp.spp; i++) {
    const size_t r = size_t(i) * n_pix + id, o = (size_t(y) * cp.w + x) * cp.spp + i;
    const CalPath& P = rec[r];
    for (uint32_t b = 0; b < CAL_MAX_DEPTH; b++) {
      tri_inst[(o * CAL_MAX_DEPTH + b) * 2] = tan[r].tri[b];
      tri_inst[(o * CAL_MAX_DEPTH + b) * 2 + 1] = tan[r].inst[b];
      for (uint32_t j = 0; j < CAL_MAX_NL; j++) q[(o * CAL_MAX_DEPTH + b) * CAL_MAX_NL + j] = b < P.n && j < cp.n_light ? P.v[b].q[j] : 0.0f;
    }
  }
}

void calib_export_paths(const CamParams& cp, const void* records, const void* tangents, uint32_t* tri_inst, float* q, cudaStream_t st) {
  const uint32_t n_pix = tiled_pixels(cp.w, cp.h, cp.tile_w, cp.tile_h);
  calib_export_paths_kernel<<<(n_pix + 127) / 128, 128, 0, st>>>(cp, static_cast<const CalPath*>(records), static_cast<const CalTan*>(tangents),
                                                                n_pix, tri_inst, q);
}

void launch_direct_transfer(const Scene& S, const float* centres, const float* normals, uint32_t n, uint32_t n_lamps, uint32_t samples, float* D,
                            cudaStream_t st) {
  const size_t total = size_t(n) * n_lamps;
  const uint32_t grid = uint32_t(std::min<size_t>((total + 127) / 128, 65535));
  direct_transfer_kernel<<<grid, 128, 0, st>>>(S, centres, normals, n, n_lamps, samples, D);
}

void launch_dl(const float* D, const float* L, uint32_t n, uint32_t n_lamps, float* y, cudaStream_t st) {
  dl_kernel<<<(n + 7) / 8, 256, 0, st>>>(D, L, n, n_lamps, y);
}

size_t jacobi_t_work(uint32_t n) { return size_t(JT_SPLITS) * n * 8; }

void launch_jacobi_t(const float* F, const double* g, const float* rho, const double* lam_in, double* lam_out, uint32_t n, double* work,
                     cudaStream_t st) {
  jacobi_t_kernel<<<dim3((n + JT_COLS - 1) / JT_COLS, JT_SPLITS), JT_COLS, 0, st>>>(F, g, rho, lam_in, n, work);
  jacobi_t_combine<<<(n + 255) / 256, 256, 0, st>>>(work, n, lam_out);
}

void launch_sum(const double* p, uint32_t n, double* out, cudaStream_t st) { sum_kernel<<<1, 1024, 0, st>>>(p, n, out); }

void launch_mul(const float* a, const float* b, float* y, uint32_t n, cudaStream_t st) { mul_kernel<<<(n + 255) / 256, 256, 0, st>>>(a, b, y, n); }

void launch_radiosity64(const float* F, const float* rho, const float* DL, uint32_t n, uint32_t iters, void* work, float* H,
                        cudaStream_t st) {
  // the three channels' iterates as float pairs, two planar 3 x n arrays in `work`
  float2* p0 = static_cast<float2*>(work);
  float2* p1 = p0 + size_t(3) * n;
  radiosity64_init<<<(3 * n + 255) / 256, 256, 0, st>>>(rho, DL, p0, n);
  float2 *cur = p0, *nxt = p1;
  for (uint32_t it = 0; it < iters; it++) {
    radiosity64_kernel<<<(n + 7) / 8, 256, 0, st>>>(F, rho, DL, cur, nxt, nullptr, n);
    std::swap(cur, nxt);
  }
  radiosity64_kernel<<<(n + 7) / 8, 256, 0, st>>>(F, rho, DL, cur, nullptr, H, n);
}

}  // namespace vtk
