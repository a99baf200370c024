// The twin's node radiosity on the device (gpu/wgsl/kernels.wgsl.js:255-461): the gather table, the direct light of
// the nodes, and the Jacobi steps of the separable node transport. Nodes are the static vertices (verts[2i] = position
// | mesh bits, verts[2i+1] = normal | area); the node state is 4 float4 per node: E_free|V, Ls slot 1, Ls slot 2,
// B_dir|vis (gpu/renderer.js:316-326).
//
// Layout in HBM: gtable u32[n_nodes x K] node-major (the K rays of a node are contiguous, so a warp reads a node's
// row in one or two coalesced transactions), aux float4[n_nodes] (escapes after the build, then one gather result
// per active node), active u32[n_active] ascending, nbr uint2[n_active x nbr_k] (active index, weight bits).
// The gather kernel runs one warp per active node: a lane takes rays j = lane, lane + 32, ... and the warp adds
// its terms by shuffles. A(mu_in) of ray j depends only on the node's material, so it comes from a per-material
// table (n_mat x K) built once per table build instead of two albedo-table lerps per ray.
#include "vt_kernels.cuh"
#include "vt_nodes.cuh"

#ifndef VT_NODE_TRACE_BLOCKS
#define VT_NODE_TRACE_BLOCKS 4   // blocks of 256 per SM the persistent shadow lanes are compiled for (64 registers)
#endif

namespace vtk {

using namespace vtd;

// gpu/wgsl/kernels.wgsl.js:271 gatherDir: K cosine-distributed rays (Fibonacci spiral on the disk, rotated per node).
// The spiral's angle fraction is rounded after each product and sum (like the Kronecker numbers), so the CPU
// restatement draws the same directions.
__device__ __forceinline__ float3 gather_dir(uint32_t i, uint32_t j, uint32_t K, float3 n) {
  const float3 t = basis_t(n), b = basis_b(n);
  const float rot = u01(pcg(i * 2654435761u + 17u));
  const float rr = sqrtf(__fdiv_rn(float(j) + 0.5f, float(K)));
  const float a = __fadd_rn(__fmul_rn(float(j), GOLD), rot);
  const float ph = 2.0f * PI_F * (a - floorf(a));
  float sn, cs;
  sincosf(ph, &sn, &cs);
  return normalize(t * (rr * cs) + b * (rr * sn) + n * sqrtf(fmaxf(0.0f, 1.0f - rr * rr)));
}
__device__ __forceinline__ float3 node_pos(const Scene& S, uint32_t i) { return xyz(__ldg(S.verts + 2u * i)); }
__device__ __forceinline__ float3 node_nrm(const Scene& S, uint32_t i) { return normalize(xyz(__ldg(S.verts + 2u * i + 1u))); }
__device__ __forceinline__ uint32_t node_mat(const Scene& S, uint32_t i) {
  return fu(__ldg(S.params + S.mesh_off + 2u * fu(__ldg(S.verts + 2u * i).w)).w);
}

// the node that hit h lands on: the hit triangle's vertex of largest barycentric, if the ray meets its front
__device__ __forceinline__ uint32_t landing_node(const Scene& S, const Hit& h, float3 dir) {
  if (h.tri == MISS) return MISS;
  const float3 bb = f3(1.0f - h.u - h.v, h.u, h.v);
  const float4* r = S.tris + 4u * h.tri;
  const uint32_t v0 = fu(__ldg(r).w), v1 = fu(__ldg(r + 1).w), v2 = fu(__ldg(r + 2).w);
  const float3 nv = xyz(__ldg(S.verts + 2u * v0 + 1u)) * bb.x + xyz(__ldg(S.verts + 2u * v1 + 1u)) * bb.y + xyz(__ldg(S.verts + 2u * v2 + 1u)) * bb.z;
  if (!(dot(nv, dir) < 0.0f)) return MISS;
  if (bb.x >= bb.y && bb.x >= bb.z) return v0;
  return bb.y >= bb.z ? v1 : v2;
}

// The gather table's rays (node i, ray j at r = i K + j) on persistent closest-hit lanes (trace_step: one node visit
// or triangle test per lane step, the same per-ray sequence as trace_scene's static descent, so the same hits); a
// lane takes the next ray when its own finishes. `head` counts the rays taken.
__global__ void __launch_bounds__(256, VT_NODE_TRACE_BLOCKS) gather_build_kernel(const Scene S, uint32_t K, uint64_t r0, uint32_t total,
                                                                                 uint32_t* __restrict__ gtable, uint32_t* head) {
  __shared__ uint2 stack_sh[SH_DEPTH * 256];
  LaneStack stk;
  stk.sh = stack_sh; stk.lane = threadIdx.x; stk.stride = 256;
  TraceState st;
  float3 o = f3(0, 0, 0), d = f3(0, 0, 1);
  uint64_t r = 0;
  bool active = false, exhausted = false;
  auto finish = [&]() {
    gtable[r] = landing_node(S, st.best, d);
    active = false;
  };
  auto start = [&](uint32_t idx) {
    r = r0 + idx;
    const uint32_t i = uint32_t(r / K), j = uint32_t(r % K);
    const float3 p = node_pos(S, i), n = node_nrm(S, i);
    d = gather_dir(i, j, K, n);
    o = p + n * EPS_OFF;
    st.best = Hit{BIG, 0.0f, 0.0f, MISS, MISS};
    active = trace_phase(S, 0u, o, d, 0.0f, 0.5f, 1u, 0u, st, -1);
    if (!active) { active = true; finish(); }
  };
  while (take_rays(active, exhausted, head, total, 8u, start)) {
    if (!active) continue;
    if (trace_step<false>(S, 0.0f, st, stk) != 0) finish();
  }
}

// escapes per node (gpu/wgsl/kernels.wgsl.js:326 gatherCount)
__global__ void gather_count_kernel(uint32_t n_nodes, uint32_t K, const uint32_t* __restrict__ gtable, float4* __restrict__ aux) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes; i += gridDim.x * blockDim.x) {
    uint32_t m = 0;
    for (uint32_t j = 0; j < K; j++) m += gtable[size_t(i) * K + j] == MISS;
    aux[i] = make_float4(float(m), 0.0f, 0.0f, 0.0f);
  }
}

// entries that point at an inactive node go to the hit triangle's active vertex of largest barycentric, if any
// (gpu/wgsl/kernels.wgsl.js:300 gatherRemap)
__global__ void gather_remap_kernel(const Scene S, uint32_t n_nodes, uint32_t K, uint32_t* __restrict__ gtable, const float4* __restrict__ aux) {
  const size_t total = size_t(n_nodes) * K;
  const float half = 0.5f * float(K);
  for (size_t r = size_t(blockIdx.x) * blockDim.x + threadIdx.x; r < total; r += size_t(gridDim.x) * blockDim.x) {
    const uint32_t v0 = gtable[r];
    if (v0 == MISS || aux[v0].x <= half) continue;
    const uint32_t i = uint32_t(r / K), j = uint32_t(r % K);
    const float3 p = node_pos(S, i), n = node_nrm(S, i);
    const float3 dir = gather_dir(i, j, K, n);
    const Hit h = trace_scene<false>(S, 0u, p + n * EPS_OFF, dir, 0.0f, BIG, 0.5f, 1u, 0u);
    if (h.tri == MISS) continue;
    const float3 bb = f3(1.0f - h.u - h.v, h.u, h.v);
    const float4* t = S.tris + 4u * h.tri;
    const uint32_t a = fu(__ldg(t).w), b = fu(__ldg(t + 1).w), c = fu(__ldg(t + 2).w);
    uint32_t best = v0;
    float bw = -1.0f;
    if (aux[a].x <= half && bb.x > bw) { best = a; bw = bb.x; }
    if (aux[b].x <= half && bb.y > bw) { best = b; bw = bb.y; }
    if (aux[c].x <= half && bb.z > bw) { best = c; bw = bb.z; }
    gtable[r] = best;
  }
}

// A(mu_in of ray j) per material: amu[m * K + j] (the table the gather kernel reads)
__global__ void amu_kernel(const Scene S, uint32_t n_mat, uint32_t K, float4* __restrict__ amu) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_mat * K; k += gridDim.x * blockDim.x) {
    const uint32_t m = k / K, j = k % K;
    const float mu = sqrtf(fmaxf(0.0f, 1.0f - __fdiv_rn(float(j) + 0.5f, float(K))));
    const float3 a = albedo(S, m, mu);
    amu[k] = make_float4(a.x, a.y, a.z, 0.0f);
  }
}

// gpu/wgsl/kernels.wgsl.js:348 nodeDirect: direct irradiance at each active node from node_samples emitter samples
// (shadow rays through the whole scene at mid-exposure), its first reflection B_dir = sum E_s A(mu_s), the
// visibility code (1 all lit samples visible, 0 none, 0.5 mixed, -1 no lit sample) and the capsule visibility V.
// moved != 0: only nodes whose segment to the emitter passes near a moved body's bounding capsule, now or at the
// last full update.
//
// In three passes, so that the shadow rays run on persistent traversal lanes: node_direct_setup (one thread per
// (node, sample): the sample, its unshadowed term and its shadow ray, queued when the sample is lit),
// node_direct_shadow (any hit of the queued rays) and node_direct_sum (per node: the visible terms added in sample
// order, the codes). Every value is the one-pass estimator's: the shadow answers do not depend on the order rays are
// traced in, and each node's terms are added in sample order.
namespace {
constexpr uint32_t ND_LIT = 1u, ND_VIS = 2u, ND_RUN = 4u;

// append `want` lanes' items to a queue with one atomic per warp; returns the slot of this lane (if want)
__device__ __forceinline__ uint32_t node_append(uint32_t* count, bool want) {
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
}  // namespace

__global__ void __launch_bounds__(256) node_direct_setup(const Scene S, const uint32_t* __restrict__ active, uint32_t n_active, uint32_t NS,
                                                         uint32_t moved, NodeDirectBufs b) {
  const float area = __ldg(S.su + 3);
  const size_t total = size_t(n_active) * NS;
  for (size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += size_t(gridDim.x) * blockDim.x) {
    const uint32_t k = uint32_t(t / NS), s = uint32_t(t % NS);
    const uint32_t i = active[k];
    const float3 p = node_pos(S, i), n = node_nrm(S, i);
    bool run = true;
    if (moved) {
      Rot R;
      float3 pp;
      inst_pose(S, ldu(S.su + 17), 0.5f, R, pp);
      const float3 dE = (rmul(R, ld3(S.su + 20)) + pp) - p;
      const float rr = __ldg(S.su + 23) + 1e-3f;
      bool near = false;
      const uint32_t cnt = min(ldu(S.su + 16), uint32_t(VT_MAX_INST));
      for (uint32_t bb = 0; bb < cnt && !near; bb++) {
        if (!((moved >> bb) & 1u)) continue;
        const float* I = inst_rec(S, bb);
        near = seg_near_capsule(p, dE, 0.0f, 1.0f, ld3(I + 32), ld3(I + 36), __ldg(I + 35) + rr) ||
               seg_near_capsule(p, dE, 0.0f, 1.0f, ld3(I + 40), ld3(I + 44), __ldg(I + 43) + rr);
      }
      run = near;
    }
    uint32_t flags = run ? ND_RUN : 0u;
    float3 c = f3(0, 0, 0);
    if (run) {
      const uint32_t hs = pcg(i * 2246822519u + 3u);
      const float s0 = u01(pcg(hs)), s1 = u01(pcg(hs + 1u)), s2 = u01(pcg(hs + 2u));
      float3 lp, ln, la;
      sample_emitter(S, f3(kr(s, KL0, s0), kr(s, KL1, s1), kr(s, KL2, s2)), 0.5f, lp, ln, la);
      float3 wi = lp - p;
      const float d2 = dot(wi, wi), dist = sqrtf(d2);
      wi = wi / dist;
      const float cosE = dot(-wi, ln), cosN = dot(n, wi);
      if (cosE > 0.0f && cosN > 0.0f) {
        const float3 Le = emitted(S, ln, la, -wi);
        if (maxc(Le) > 0.0f) {
          flags |= ND_LIT;
          c = Le * (cosE * cosN * area / d2) * albedo(S, node_mat(S, i), cosN);
          const float3 o = p + n * EPS_OFF;
          b.ro[t] = make_float4(o.x, o.y, o.z, dist - 2e-5f);
          b.rd[t] = make_float4(wi.x, wi.y, wi.z, 0.0f);
        }
      }
    }
    b.term[t] = make_float4(c.x, c.y, c.z, __uint_as_float(flags));
    const uint32_t q = node_append(b.counts, (flags & ND_LIT) != 0u);
    if (flags & ND_LIT) b.queue[q] = uint32_t(t);
  }
}

// any hit of every queued shadow ray (the static BVH, then each posed body that passes its culls) on persistent
// lanes; a visible sample gets ND_VIS
__global__ void __launch_bounds__(256, VT_NODE_TRACE_BLOCKS) node_direct_shadow(const Scene S, NodeDirectBufs b, uint32_t refill) {
  const uint32_t n = b.counts[0];
  const uint32_t skip = ldu(S.su + 7);
  __shared__ uint2 stack_sh[SH_DEPTH * 256];
  LaneStack stk;
  stk.sh = stack_sh; stk.lane = threadIdx.x; stk.stride = 256;
  TraceState st;
  float3 o = f3(0, 0, 0), d = f3(0, 0, 1);
  uint32_t t = 0;
  bool active = false, exhausted = false;
  auto visible = [&]() { b.term[t].w = __uint_as_float(__float_as_uint(b.term[t].w) | ND_VIS); };
  auto start = [&](uint32_t idx) {
    t = b.queue[idx];
    const float4 o4 = b.ro[t], d4 = b.rd[t];
    o = xyz(o4); d = xyz(d4);
    st.best = Hit{o4.w, 0.0f, 0.0f, MISS, MISS};
    active = trace_phase(S, 0u, o, d, 0.0f, 0.5f, 3u, skip, st, -1);
    if (!active) visible();
  };
  while (take_rays(active, exhausted, b.counts + 1, n, refill, start)) {
    if (!active) continue;
    const int r = trace_step<true>(S, 0.0f, st, stk);
    bool done = r == 2;
    if (r == 1) done = !trace_phase(S, 0u, o, d, 0.0f, 0.5f, 3u, skip, st, st.k + 1);
    if (!done) continue;
    if (st.best.tri == MISS) visible();
    active = false;
  }
}

__global__ void node_direct_sum(const Scene S, const uint32_t* __restrict__ active, uint32_t n_active, uint32_t NS, NodeDirectBufs b,
                                float4* __restrict__ nstate) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_active; k += gridDim.x * blockDim.x) {
    const size_t t0 = size_t(k) * NS;
    if (!(__float_as_uint(b.term[t0].w) & ND_RUN)) continue;
    float3 B = f3(0, 0, 0);
    uint32_t n_lit = 0, n_vis = 0;
    for (uint32_t s = 0; s < NS; s++) {
      const float4 c = b.term[t0 + s];
      const uint32_t f = __float_as_uint(c.w);
      n_lit += (f & ND_LIT) ? 1u : 0u;
      if (f & ND_VIS) { n_vis++; B = B + xyz(c); }
    }
    B = B / float(NS);
    const uint32_t i = active[k];
    const float vis = n_lit == 0 ? -1.0f : n_vis == n_lit ? 1.0f : n_vis == 0 ? 0.0f : 0.5f;
    nstate[4u * i + 3u] = make_float4(B.x, B.y, B.z, vis);
    const float4 old = nstate[4u * i];
    nstate[4u * i] = make_float4(old.x, old.y, old.z, capsule_vis(S, node_pos(S, i), node_nrm(S, i)));
  }
}

// jacobiGather (gpu/wgsl/kernels.wgsl.js:416): aux[k] = (pi / K) sum_j A_i(mu_in_j) A_h(mu_out_j) Ls_h / hh_i over
// the rays that land on a node h. One warp per active node.
__global__ void __launch_bounds__(256) jacobi_gather_kernel(const Scene S, const uint32_t* __restrict__ active, uint32_t n_active, uint32_t K,
                                                            const uint32_t* __restrict__ gtable, const float4* __restrict__ amu,
                                                            uint32_t slot_in, const float4* __restrict__ nstate, float4* __restrict__ aux) {
  const uint32_t lane = threadIdx.x & 31u;
  for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n_active; k += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t i = active[k];
    const float3 n = node_nrm(S, i);
    const uint32_t mi = node_mat(S, i);
    float3 acc = f3(0, 0, 0);
    for (uint32_t j = lane; j < K; j += 32) {
      const uint32_t h = gtable[size_t(i) * K + j];
      if (h == MISS) continue;
      const float3 dir = gather_dir(i, j, K, n);
      const float mu_out = clampf(-dot(dir, node_nrm(S, h)), 0.0f, 1.0f);
      acc = acc + xyz(__ldg(amu + mi * K + j)) * albedo(S, node_mat(S, h), mu_out) * xyz(nstate[4u * h + slot_in]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
      acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
    }
    if (lane == 0) {
      const float4* M = S.params + S.mat_off + 5u * mi;
      const float3 hh = xyz(__ldg(M + 2));
      const float sc = PI_F / float(K);
      aux[k] = make_float4(acc.x * sc / fmaxf(hh.x, 1e-4f), acc.y * sc / fmaxf(hh.y, 1e-4f), acc.z * sc / fmaxf(hh.z, 1e-4f), 0.0f);
    }
  }
}

// jacobiUpdate (gpu/wgsl/kernels.wgsl.js:440): E_free = weighted mean of aux over the node's neighbours, and the
// separable source Ls = (B_dir + E_free V hh) / (pi hh) into slot_out (w = 1 marks a solved node)
__global__ void jacobi_update_kernel(const Scene S, const uint32_t* __restrict__ active, uint32_t n_active, const uint2* __restrict__ nbr,
                                     uint32_t nbr_k, const float4* __restrict__ aux, uint32_t slot_out, float4* __restrict__ nstate) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_active; k += gridDim.x * blockDim.x) {
    const uint32_t i = active[k];
    float3 ef = f3(0, 0, 0);
    float ws = 0.0f;
    for (uint32_t j = 0; j < nbr_k; j++) {
      const uint2 e = __ldcs(nbr + size_t(k) * nbr_k + j);
      const float w = __uint_as_float(e.y);
      if (w <= 0.0f) break;
      ef = ef + xyz(aux[e.x]) * w;
      ws += w;
    }
    ef = ws > 0.0f ? ef / ws : xyz(aux[k]);
    const float4 st = nstate[4u * i];
    const float4* M = S.params + S.mat_off + 5u * node_mat(S, i);
    const float3 hh = xyz(__ldg(M + 2));
    const float3 hm = f3(fmaxf(hh.x, 1e-4f), fmaxf(hh.y, 1e-4f), fmaxf(hh.z, 1e-4f));
    const float3 bd = xyz(nstate[4u * i + 3u]);
    const float3 L = f3((bd.x + ef.x * st.w * hm.x) * INV_PI_F / hm.x, (bd.y + ef.y * st.w * hm.y) * INV_PI_F / hm.y,
                        (bd.z + ef.z * st.w * hm.z) * INV_PI_F / hm.z);
    nstate[4u * i] = make_float4(ef.x, ef.y, ef.z, st.w);
    nstate[4u * i + slot_out] = make_float4(L.x, L.y, L.z, 1.0f);
  }
}

// ------------------------------------------------------------------------------------------------ transport table
// The gather's per-ray factor (pi / K) A_i(mu_in_j) A_h(mu_out_j) / hh_i depends only on the static geometry and
// the materials, so it is evaluated once per table build into a compressed row per active node: one float4 per
// landing ray (weight rgb, node bits), rays in index order, escapes dropped. A Jacobi gather is then a sparse
// matrix-vector product: one coalesced 16-byte load per entry plus the landing node's Ls (L2-resident).
__global__ void transport_count_kernel(const uint32_t* __restrict__ active, uint32_t n_active, uint32_t K, const uint32_t* __restrict__ gtable,
                                       uint32_t* __restrict__ cnt) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_active; k += gridDim.x * blockDim.x) {
    const uint32_t i = active[k];
    uint32_t c = 0;
    for (uint32_t j = 0; j < K; j++) c += gtable[size_t(i) * K + j] != MISS;
    cnt[k] = c;
  }
}

__global__ void __launch_bounds__(256) transport_fill_kernel(const Scene S, const uint32_t* __restrict__ active, uint32_t n_active, uint32_t K,
                                                             const uint32_t* __restrict__ gtable, const float4* __restrict__ amu,
                                                             const uint32_t* __restrict__ row, float4* __restrict__ ent) {
  const uint32_t lane = threadIdx.x & 31u;
  for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n_active; k += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t i = active[k];
    const float3 n = node_nrm(S, i);
    const uint32_t mi = node_mat(S, i);
    const float3 hh = xyz(__ldg(S.params + S.mat_off + 5u * mi + 2u));
    const float sc = PI_F / float(K);
    const float3 f = f3(sc / fmaxf(hh.x, 1e-4f), sc / fmaxf(hh.y, 1e-4f), sc / fmaxf(hh.z, 1e-4f));
    uint32_t base = row[k];
    for (uint32_t j0 = 0; j0 < K; j0 += 32) {
      const uint32_t j = j0 + lane;
      const uint32_t h = j < K ? gtable[size_t(i) * K + j] : MISS;
      const bool valid = h != MISS;
      const uint32_t m = __ballot_sync(0xffffffffu, valid);
      if (valid) {
        const float3 dir = gather_dir(i, j, K, n);
        const float mu_out = clampf(-dot(dir, node_nrm(S, h)), 0.0f, 1.0f);
        const float3 w = xyz(__ldg(amu + mi * K + j)) * albedo(S, node_mat(S, h), mu_out) * f;
        ent[base + __popc(m & ((1u << lane) - 1u))] = make_float4(w.x, w.y, w.z, __uint_as_float(h));
      }
      base += __popc(m);
    }
  }
}

// jacobiGather over the transport table: aux[k] = sum over the row of weight x Ls_h. A half-warp per row, four
// 16-byte entries per lane in flight (a row of K = 64 rays in one pass), then the landing nodes' Ls; the entry
// stream is the only DRAM traffic that grows with the rays; it is loaded evict-first, so the node state (21 MB at
// 331k nodes) stays in L2 for the gathers.
__global__ void __launch_bounds__(256) jacobi_gather_table_kernel(const uint32_t* __restrict__ row, const float4* __restrict__ ent, uint32_t n_active,
                                                                  uint32_t slot_in, const float4* __restrict__ nstate, float4* __restrict__ aux) {
  const uint32_t hl = threadIdx.x & 15u;
  const uint32_t half = (blockIdx.x * blockDim.x + threadIdx.x) >> 4, halves = (gridDim.x * blockDim.x) >> 4;
  // whole warps iterate together (the half-warp shuffles need both halves present)
  const uint32_t rounds = (n_active + halves - 1) / halves;
  for (uint32_t it = 0; it < rounds; it++) {
    const uint32_t k = half + it * halves;
    const bool in = k < n_active;
    const uint32_t e0 = in ? row[k] : 0u, e1 = in ? row[k + 1] : 0u;
    float3 acc = f3(0, 0, 0);
    for (uint32_t b = e0; b < e1; b += 64) {
      float4 w[4], l[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const uint32_t e = b + hl + 16u * q;
        w[q] = e < e1 ? __ldcs(ent + e) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);   // streamed: keep Ls in L2
      }
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const uint32_t e = b + hl + 16u * q;
        l[q] = e < e1 ? nstate[4u * __float_as_uint(w[q].w) + slot_in] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
#pragma unroll
      for (int q = 0; q < 4; q++) acc = acc + xyz(w[q]) * xyz(l[q]);
    }
    for (int o = 8; o > 0; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
      acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
    }
    if (in && hl == 0) aux[k] = make_float4(acc.x, acc.y, acc.z, 0.0f);
  }
}

static int grid_for(size_t work, int threads) {
  const size_t g = (work + threads - 1) / threads;
  return int(std::max<size_t>(1, std::min<size_t>(g, 152 * 64)));
}

void launch_gather_build(const Scene& S, uint32_t n_nodes, uint32_t K, uint32_t* gtable, float4* aux, cudaStream_t st) {
  const size_t rays = size_t(n_nodes) * K;
  static std::atomic<int> grid[MAX_DEVICES];
  const int g = per_device_value(grid, [](int dev) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, gather_build_kernel, 256, 0);
    return device_sms(dev) * std::max(1, per);
  });
  // aux's first word counts the rays taken (aux is written by gather_count_kernel afterwards); at most 2^31 rays per
  // launch
  uint32_t* head = reinterpret_cast<uint32_t*>(aux);
  for (size_t r0 = 0; r0 < rays; r0 += size_t(1) << 31) {
    cudaMemsetAsync(head, 0, 4, st);
    gather_build_kernel<<<g, 256, 0, st>>>(S, K, r0, uint32_t(std::min(rays - r0, size_t(1) << 31)), gtable, head);
  }
  gather_count_kernel<<<grid_for(n_nodes, 128), 128, 0, st>>>(n_nodes, K, gtable, aux);
  gather_remap_kernel<<<grid_for(rays, 128), 128, 0, st>>>(S, n_nodes, K, gtable, aux);
}

void launch_amu(const Scene& S, uint32_t n_mat, uint32_t K, float4* amu, cudaStream_t st) {
  amu_kernel<<<grid_for(size_t(n_mat) * K, 128), 128, 0, st>>>(S, n_mat, K, amu);
}

size_t node_direct_bytes(uint32_t n_active, uint32_t NS) { return size_t(n_active) * NS * (3 * 16 + 4) + 256; }

void launch_node_direct(const Scene& S, const uint32_t* active, uint32_t n_active, uint32_t NS, uint32_t moved, float4* nstate, void* work,
                        int trace_blocks, cudaStream_t st) {
  if (!n_active) return;
  const size_t total = size_t(n_active) * NS;
  char* w = static_cast<char*>(work);
  NodeDirectBufs b;
  b.counts = reinterpret_cast<uint32_t*>(w);
  b.ro = reinterpret_cast<float4*>(w + 256);
  b.rd = b.ro + total;
  b.term = b.rd + total;
  b.queue = reinterpret_cast<uint32_t*>(b.term + total);
  cudaMemsetAsync(b.counts, 0, 8, st);
  node_direct_setup<<<grid_for(total, 256), 256, 0, st>>>(S, active, n_active, NS, moved, b);
  node_direct_shadow<<<trace_blocks, 256, 0, st>>>(S, b, 8u);
  node_direct_sum<<<grid_for(n_active, 256), 256, 0, st>>>(S, active, n_active, NS, b, nstate);
}

void launch_transport_count(const uint32_t* active, uint32_t n_active, uint32_t K, const uint32_t* gtable, uint32_t* cnt, cudaStream_t st) {
  if (!n_active) return;
  transport_count_kernel<<<grid_for(n_active, 128), 128, 0, st>>>(active, n_active, K, gtable, cnt);
}

void launch_transport_fill(const Scene& S, const uint32_t* active, uint32_t n_active, uint32_t K, const uint32_t* gtable, const float4* amu,
                           const uint32_t* row, float4* ent, cudaStream_t st) {
  if (!n_active) return;
  transport_fill_kernel<<<grid_for(size_t(n_active) * 32, 256), 256, 0, st>>>(S, active, n_active, K, gtable, amu, row, ent);
}

void launch_jacobi_step(const Scene& S, const uint32_t* active, uint32_t n_active, uint32_t K, const uint32_t* gtable, const float4* amu,
                        const uint32_t* row, const float4* ent, const uint2* nbr, uint32_t nbr_k, uint32_t slot_in, uint32_t slot_out,
                        float4* nstate, float4* aux, cudaStream_t st) {
  if (!n_active) return;
  if (ent)
    jacobi_gather_table_kernel<<<grid_for(size_t(n_active) * 16, 256), 256, 0, st>>>(row, ent, n_active, slot_in, nstate, aux);
  else
    jacobi_gather_kernel<<<grid_for(size_t(n_active) * 32, 256), 256, 0, st>>>(S, active, n_active, K, gtable, amu, slot_in, nstate, aux);
  jacobi_update_kernel<<<grid_for(n_active, 128), 128, 0, st>>>(S, active, n_active, nbr, nbr_k, aux, slot_out, nstate);
}

}  // namespace vtk
