// Binned-SAH BVH2 build on the GPU: the tree of vt::sah_build (gpu/bvh.js:18-161), word for word.
//
// The host builder decides each node from its slot range alone. It computes the range's bounds, bins the
// centroids in 16 bins per axis, takes the cheapest SAH split (traversal and intersection cost 1), and partitions
// the slot order in place with gpu/bvh.js's swap-with-the-end loop. The nodes are then numbered in LIFO task
// order. Here every level of the tree is one pass over its tasks. A task of at least BIG_TASK slots gets a
// 512-thread block, a smaller one a warp. The task computes bounds, bins, SAH choice and partition, then appends
// its two children to the next level. The host replays the LIFO numbering over the decided shapes, so the node
// array is the host builder's.
//
// Exactness:
// - Bounds and per-bin bounds are minima and maxima of floats, exact in any order. A node box keeps the first slot
//   among equal values, as the host's strict comparisons do: the keys carry the slot, so -0 and +0 keep the host's
//   choice.
// - Bin indices and SAH costs use the host's double arithmetic, compiled without contraction.
// - The partition is the closed form of the swap-with-the-end loop over the range [s, e) with m0 = s + (number of
//   left slots). The left part [s, m0) keeps its left slots. Its k-th right slot takes the place of the k-th left
//   slot of [m0, e) counted from the top (position q_k) and moves to q_{k-1} - 1, with q_0 = e. A right slot x of
//   [m0, e) moves to x - 1, except x = m0, which moves to q_K - 1.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "vt_host.h"

namespace vtk {
namespace {

constexpr int BINS = 16;
#ifndef VT_BVH_BLOCK
#define VT_BVH_BLOCK 512
#endif
#ifndef VT_BVH_BIG
#define VT_BVH_BIG 8192
#endif
constexpr int BT = VT_BVH_BLOCK;   // threads of a big task's block
constexpr int BIG_TASK = VT_BVH_BIG;   // ranges of at least this many slots are big tasks
constexpr int WPB = 8;             // warp tasks per 256-thread block
constexpr double KBIG = 1e30;
constexpr int THR_MIN = 64;        // ranges above this many slots bin through float thresholds

struct Task { int32_t s, e, parent, slot; };
struct Shape { int32_t s, e, m, child[2]; float lo[2][3], hi[2][3]; };

struct Build {
  const float4 *bmin, *bmax, *cen;   // per triangle: box and centroid (xyz)
  uint32_t *order, *scratch;
  int32_t* qpos;
  Shape* shapes;
  uint32_t* counters;                // [0] shapes, [1] next big tasks, [2] next small tasks
  Task *next_big, *next_small;
  float* root_box;                   // lo xyz, hi xyz of the whole range
  int32_t* root_leaf;
  uint32_t leaf;
};

// per-group shared state
struct GroupSh {
  uint32_t cnt[3][BINS];
  uint32_t blo[3][BINS][3], bhi[3][BINS][3];   // order-preserving float keys
  unsigned long long red64[BT / 32];
  float redf[BT / 32];
  uint32_t redu[BT / 32];
  int32_t dec[4];                    // axis, bin, split
  double origin, scale;
  float thr[3][BINS - 1];            // per axis the least centroid of bins 1..15
};

__device__ __forceinline__ uint32_t ord(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord(uint32_t u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }
__device__ __forceinline__ float comp(const float4& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

template <int G>
struct Grp {
  int lane, warp;
  GroupSh* sh;
  __device__ __forceinline__ void sync() const {
    if (G == 32) __syncwarp(); else __syncthreads();
  }
  __device__ __forceinline__ unsigned long long min64(unsigned long long v) const {
    for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (G == 32) return v;
    __syncthreads();
    if ((lane & 31) == 0) sh->red64[warp] = v;
    __syncthreads();
    v = sh->red64[0];
    for (int i = 1; i < G / 32; i++) v = min(v, sh->red64[i]);
    return v;
  }
  __device__ __forceinline__ unsigned long long max64(unsigned long long v) const {
    for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (G == 32) return v;
    __syncthreads();
    if ((lane & 31) == 0) sh->red64[warp] = v;
    __syncthreads();
    v = sh->red64[0];
    for (int i = 1; i < G / 32; i++) v = max(v, sh->red64[i]);
    return v;
  }
  __device__ __forceinline__ float minf(float v) const {
    for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (G == 32) return v;
    __syncthreads();
    if ((lane & 31) == 0) sh->redf[warp] = v;
    __syncthreads();
    v = sh->redf[0];
    for (int i = 1; i < G / 32; i++) v = fminf(v, sh->redf[i]);
    return v;
  }
  __device__ __forceinline__ float maxf(float v) const {
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (G == 32) return v;
    __syncthreads();
    if ((lane & 31) == 0) sh->redf[warp] = v;
    __syncthreads();
    v = sh->redf[0];
    for (int i = 1; i < G / 32; i++) v = fmaxf(v, sh->redf[i]);
    return v;
  }
  __device__ __forceinline__ uint32_t sum(uint32_t v) const {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (G == 32) return v;
    __syncthreads();
    if ((lane & 31) == 0) sh->redu[warp] = v;
    __syncthreads();
    v = 0;
    for (int i = 0; i < G / 32; i++) v += sh->redu[i];
    return v;
  }
  // exclusive rank of this thread among the flagged ones of the group, and their total
  __device__ __forceinline__ uint32_t scan(bool f, uint32_t& total) const {
    const uint32_t b = __ballot_sync(0xffffffffu, f);
    const uint32_t l = lane & 31;
    const uint32_t ex = __popc(b & ((1u << l) - 1u));
    if (G == 32) { total = __popc(b); return ex; }
    __syncthreads();
    if (l == 0) sh->redu[warp] = __popc(b);
    __syncthreads();
    uint32_t off = 0, tot = 0;
    for (int i = 0; i < G / 32; i++) { const uint32_t v = sh->redu[i]; if (i < warp) off += v; tot += v; }
    total = tot;
    return off + ex;
  }
};

// std::max(0.0, d) keeps +0 for d = -0, which fmax need not
__device__ __forceinline__ double pos0(double d) { return 0.0 < d ? d : 0.0; }
__device__ __forceinline__ double half_area(const double* lo, const double* hi) {
  const double x = pos0(hi[0] - lo[0]), y = pos0(hi[1] - lo[1]), z = pos0(hi[2] - lo[2]);
  return x * y + y * z + z * x;
}
__device__ __forceinline__ int bin_of(float c, double origin, double scale) {
  const long long b = (long long)floor((double(c) - origin) * scale);
  return b >= BINS ? BINS - 1 : int(b);
}
// The least float c whose bin index floor((double(c) - origin) * scale) is at least b. The index does not decrease
// with c, so bin_of(c) = #{b in 1..15 : c >= threshold_b}, the same bin from float compares. The estimate
// origin + b / scale is within a few ulps; a search over the float order settles anything farther.
__device__ float bin_threshold(double origin, double scale, int b) {
  auto reach = [&](float c) { return (double(c) - origin) * scale >= double(b); };
  float c = float(origin + double(b) / scale);
  for (int i = 0; i < 8; i++) {
    if (reach(c)) {
      const float d = unord(ord(c) - 1u);
      if (!reach(d)) return c;
      c = d;
    } else {
      c = unord(ord(c) + 1u);
    }
  }
  uint32_t lo = ord(-INFINITY), hi = ord(INFINITY);   // reach(lo) false, reach(hi) true
  while (hi - lo > 1u) {
    const uint32_t mid = lo + (hi - lo) / 2u;
    if (reach(unord(mid))) hi = mid; else lo = mid;
  }
  return unord(hi);
}
__device__ __forceinline__ int bin_by_threshold(const float* t, float c) {
  int b = 0;
  for (int step = 8; step; step >>= 1)
    if (b + step <= BINS - 1 && c >= t[b + step - 1]) b += step;
  return b;
}

// one task: bounds, SAH choice, partition, children
template <int G>
__device__ void run_task(const Build& B, const Task T, const Grp<G>& g) {
  GroupSh& sh = *g.sh;
  const int32_t s = T.s, e = T.e, cnt = e - s;
  // bounds: node box with the first slot among equal values, centroid box plain
  unsigned long long klo[3], khi[3];
  float clo[3], chi[3];
  for (int k = 0; k < 3; k++) { klo[k] = ~0ull; khi[k] = 0ull; clo[k] = INFINITY; chi[k] = -INFINITY; }
  for (int32_t p = s + g.lane; p < e; p += G) {
    const uint32_t t = B.order[p];
    const float4 a = B.bmin[t], z = B.bmax[t], c = B.cen[t];
    const uint32_t off = uint32_t(p - s);
    for (int k = 0; k < 3; k++) {
      const float av = comp(a, k), zv = comp(z, k);
      const unsigned long long ka = (static_cast<unsigned long long>(ord(av == 0.0f ? 0.0f : av)) << 32) | off;
      const unsigned long long kz = (static_cast<unsigned long long>(ord(zv == 0.0f ? 0.0f : zv)) << 32) | (0xffffffffu - off);
      klo[k] = min(klo[k], ka);
      khi[k] = max(khi[k], kz);
      clo[k] = fminf(clo[k], comp(c, k));
      chi[k] = fmaxf(chi[k], comp(c, k));
    }
  }
  for (int k = 0; k < 3; k++) {
    klo[k] = g.min64(klo[k]); khi[k] = g.max64(khi[k]);
    clo[k] = g.minf(clo[k]); chi[k] = g.maxf(chi[k]);
  }
  if (g.lane == 0) {
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
      lo[k] = comp(B.bmin[B.order[s + uint32_t(klo[k] & 0xffffffffu)]], k);
      hi[k] = comp(B.bmax[B.order[s + (0xffffffffu - uint32_t(khi[k] & 0xffffffffu))]], k);
    }
    if (T.parent >= 0) {
      Shape& P = B.shapes[T.parent];
      for (int k = 0; k < 3; k++) { P.lo[T.slot][k] = lo[k]; P.hi[T.slot][k] = hi[k]; }
    } else {
      for (int k = 0; k < 3; k++) { B.root_box[k] = lo[k]; B.root_box[3 + k] = hi[k]; }
    }
  }
  if (cnt <= 1) {
    if (g.lane == 0 && T.parent < 0) *B.root_leaf = 1;
    return;
  }
  // bins per axis with a positive centroid extent
  double origin[3], scale[3];
  bool use[3];
  for (int k = 0; k < 3; k++) {
    origin[k] = double(clo[k]);
    const double extent = double(chi[k]) - origin[k];
    use[k] = extent > 0;
    scale[k] = use[k] ? BINS / extent : 0.0;
  }
  // FP64 is a small fraction of FP32 on this part: a range of more than THR_MIN slots bins its centroids through
  // each axis' 15 float thresholds (bin_threshold) instead of one double expression per slot and axis
  const bool thr = cnt > THR_MIN;
  for (int i = g.lane; i < 3 * BINS; i += G) {
    (&sh.cnt[0][0])[i] = 0;
    for (int k = 0; k < 3; k++) { (&sh.blo[0][0][0])[3 * i + k] = 0xffffffffu; (&sh.bhi[0][0][0])[3 * i + k] = 0u; }
    if (thr && i < 3 * (BINS - 1)) {
      const int ax = i / (BINS - 1), b = i % (BINS - 1) + 1;
      sh.thr[ax][b - 1] = use[ax] ? bin_threshold(origin[ax], scale[ax], b) : INFINITY;
    }
  }
  g.sync();
  for (int32_t p = s + g.lane; p < e; p += G) {
    const uint32_t t = B.order[p];
    const float4 a = B.bmin[t], z = B.bmax[t], c = B.cen[t];
    for (int ax = 0; ax < 3; ax++) {
      if (!use[ax]) continue;
      const int b = thr ? bin_by_threshold(sh.thr[ax], comp(c, ax)) : bin_of(comp(c, ax), origin[ax], scale[ax]);
      atomicAdd(&sh.cnt[ax][b], 1u);
      for (int k = 0; k < 3; k++) {
        atomicMin(&sh.blo[ax][b][k], ord(comp(a, k)));
        atomicMax(&sh.bhi[ax][b][k], ord(comp(z, k)));
      }
    }
  }
  g.sync();
  // SAH choice (gpu/bvh.js:60-118) on the group's first warp: a 16-lane segment per axis holds its bins, prefix and
  // suffix boxes come from segmented scans, and lane b prices the split after bin b. Only splits after a non-empty
  // bin are priced: the splits that follow an empty bin cost exactly what the last split after a non-empty bin
  // costs, and the host's strict comparison keeps the earlier one. The cheapest split wins, ties to the lower
  // (axis, bin), which is the host's loop order.
  if (g.lane < 32) {
    const int l16 = g.lane & 15;
    double plo[3], phi[3];
    for (int k = 0; k < 3; k++) {
      plo[k] = double(comp(B.bmin[B.order[s + uint32_t(klo[k] & 0xffffffffu)]], k));
      phi[k] = double(comp(B.bmax[B.order[s + (0xffffffffu - uint32_t(khi[k] & 0xffffffffu))]], k));
    }
    const double parent = half_area(plo, phi);
    double best_cost = INFINITY;
    int best_idx = 1 << 30;
    for (int round = 0; round < 2; round++) {
      const int ax = round * 2 + (g.lane >> 4);
      const bool live = ax < 3 && use[ax];
      const uint32_t c = live ? sh.cnt[ax][l16] : 0u;
      float lo[3], hi[3];
      for (int k = 0; k < 3; k++) {
        lo[k] = c ? unord(sh.blo[ax < 3 ? ax : 0][l16][k]) : INFINITY;
        hi[k] = c ? unord(sh.bhi[ax < 3 ? ax : 0][l16][k]) : -INFINITY;
      }
      // inclusive prefix (bins 0..b) and suffix (bins b..15) within the segment
      uint32_t pc = c, sc = c;
      float pl[3] = {lo[0], lo[1], lo[2]}, ph[3] = {hi[0], hi[1], hi[2]}, sl[3] = {lo[0], lo[1], lo[2]}, shh[3] = {hi[0], hi[1], hi[2]};
      for (int d = 1; d < 16; d <<= 1) {
        const uint32_t uc = __shfl_up_sync(0xffffffffu, pc, d, 16), dc = __shfl_down_sync(0xffffffffu, sc, d, 16);
        float ul[3], uh[3], dl[3], dh[3];
        for (int k = 0; k < 3; k++) {
          ul[k] = __shfl_up_sync(0xffffffffu, pl[k], d, 16); uh[k] = __shfl_up_sync(0xffffffffu, ph[k], d, 16);
          dl[k] = __shfl_down_sync(0xffffffffu, sl[k], d, 16); dh[k] = __shfl_down_sync(0xffffffffu, shh[k], d, 16);
        }
        if (l16 >= d) { pc += uc; for (int k = 0; k < 3; k++) { pl[k] = fminf(pl[k], ul[k]); ph[k] = fmaxf(ph[k], uh[k]); } }
        if (l16 + d < 16) { sc += dc; for (int k = 0; k < 3; k++) { sl[k] = fminf(sl[k], dl[k]); shh[k] = fmaxf(shh[k], dh[k]); } }
      }
      // the suffix of bin b + 1
      const uint32_t rc = __shfl_down_sync(0xffffffffu, sc, 1, 16);
      float rl[3], rh[3];
      for (int k = 0; k < 3; k++) { rl[k] = __shfl_down_sync(0xffffffffu, sl[k], 1, 16); rh[k] = __shfl_down_sync(0xffffffffu, shh[k], 1, 16); }
      if (live && l16 < BINS - 1 && c && rc) {
        const double la[3] = {double(pl[0]), double(pl[1]), double(pl[2])}, lb[3] = {double(ph[0]), double(ph[1]), double(ph[2])};
        const double ra[3] = {double(rl[0]), double(rl[1]), double(rl[2])}, rb[3] = {double(rh[0]), double(rh[1]), double(rh[2])};
        const double cost = 1.0 + 1.0 * (double(pc) * half_area(la, lb) + double(rc) * half_area(ra, rb)) / parent;
        if (cost < best_cost) { best_cost = cost; best_idx = ax * 16 + l16; }
      }
    }
    for (int o = 16; o; o >>= 1) {
      const double oc = __shfl_xor_sync(0xffffffffu, best_cost, o);
      const int oi = __shfl_xor_sync(0xffffffffu, best_idx, o);
      if (oc < best_cost || (oc == best_cost && oi < best_idx)) { best_cost = oc; best_idx = oi; }
    }
    if (g.lane == 0) {
      const int best_axis = best_idx < (1 << 30) ? best_idx >> 4 : -1, best_bin = best_axis >= 0 ? best_idx & 15 : -1;
      // split: -1 leaf, -2 median without partition, 0 partition at (axis, bin)
      int split = 0;
      if (best_axis < 0) split = cnt > int32_t(B.leaf) * 4 ? -2 : -1;
      else if (cnt <= int32_t(B.leaf) && best_cost >= double(cnt)) split = -1;
      sh.dec[0] = best_axis; sh.dec[1] = best_bin; sh.dec[2] = split;
      if (split == 0) { sh.origin = origin[best_axis]; sh.scale = scale[best_axis]; }
    }
  }
  g.sync();
  const int split = sh.dec[2];
  int32_t m;
  if (split == -1) {
    if (g.lane == 0 && T.parent < 0) *B.root_leaf = 1;
    return;
  } else if (split == -2) {
    m = s + (cnt >> 1);
  } else {
    const int ax = sh.dec[0], bb = sh.dec[1];
    const double o = sh.origin, sc = sh.scale;
    // left of the split: bin <= bb, i.e. below the threshold of bin bb + 1
    const float cut = thr ? sh.thr[ax][bb] : 0.0f;
    auto left = [&](uint32_t t) {
      const float c = comp(B.cen[t], ax);
      return thr ? c < cut : bin_of(c, o, sc) <= bb;
    };
    uint32_t nl = 0;
    for (int32_t p = s + g.lane; p < e; p += G) nl += left(B.order[p]) ? 1u : 0u;
    nl = g.sum(nl);
    const int32_t m0 = s + int32_t(nl);
    // [m0, e) from the top: the left slots' positions q_1 > q_2 > ... into qpos[s + k - 1]; right slots move down one
    uint32_t K = 0;
    for (int32_t base = 0; base < e - m0; base += G) {
      const int32_t x = e - 1 - (base + g.lane);
      const bool valid = x >= m0;
      const uint32_t t = valid ? B.order[x] : 0u;
      const bool L = valid && left(t);
      uint32_t tot;
      const uint32_t r = g.scan(L, tot);
      if (L) B.qpos[s + K + r] = x;
      else if (valid && x > m0) B.scratch[x - 1] = t;
      K += tot;
    }
    g.sync();
    // the lowest slot of [m0, e), when right, goes to q_K - 1
    if (g.lane == 0 && m0 < e) {
      const uint32_t t = B.order[m0];
      if (!left(t)) B.scratch[(K ? B.qpos[s + K - 1] : e) - 1] = t;
    }
    // [s, m0) from the bottom: left slots stay, the k-th right slot trades places with the k-th left slot of the top
    uint32_t k0 = 0;
    for (int32_t base = 0; base < m0 - s; base += G) {
      const int32_t p = s + base + g.lane;
      const bool valid = p < m0;
      const uint32_t t = valid ? B.order[p] : 0u;
      const bool R = valid && !left(t);
      uint32_t tot;
      const uint32_t r = g.scan(R, tot);
      if (R) {
        const uint32_t k = k0 + r + 1;   // 1-based rank among the right slots of [s, m0)
        B.scratch[(k == 1 ? e : B.qpos[s + k - 2]) - 1] = t;
        B.scratch[p] = B.order[B.qpos[s + k - 1]];
      } else if (valid) {
        B.scratch[p] = t;
      }
      k0 += tot;
    }
    g.sync();
    for (int32_t p = s + g.lane; p < e; p += G) B.order[p] = B.scratch[p];
    g.sync();
    m = (m0 == s || m0 == e) ? s + (cnt >> 1) : m0;
  }
  // an interior node: its shape, and its two children as tasks of the next level
  if (g.lane == 0) {
    const uint32_t id = atomicAdd(B.counters, 1u);
    Shape& S = B.shapes[id];
    S.s = s; S.e = e; S.m = m; S.child[0] = -1; S.child[1] = -1;
    if (T.parent >= 0) B.shapes[T.parent].child[T.slot] = int32_t(id);
    auto push = [&](const Task c) {
      if (c.e - c.s >= BIG_TASK) B.next_big[atomicAdd(B.counters + 1, 1u)] = c;
      else B.next_small[atomicAdd(B.counters + 2, 1u)] = c;
    };
    push(Task{s, m, int32_t(id), 0});
    push(Task{m, e, int32_t(id), 1});
  }
}

__global__ void __launch_bounds__(BT) big_tasks(Build B, const Task* __restrict__ tasks) {
  __shared__ GroupSh sh;
  Grp<BT> g{int(threadIdx.x), int(threadIdx.x >> 5), &sh};
  run_task<BT>(B, tasks[blockIdx.x], g);
}

__global__ void __launch_bounds__(32 * WPB) small_tasks(Build B, const Task* __restrict__ tasks, uint32_t n) {
  __shared__ GroupSh sh[WPB];
  const uint32_t w = threadIdx.x >> 5, i = blockIdx.x * WPB + w;
  if (i >= n) return;   // whole warps leave: a warp task synchronises only within its warp
  Grp<32> g{int(threadIdx.x & 31), 0, &sh[w]};
  run_task<32>(B, tasks[i], g);
}

// per triangle: its box as the host builder takes it (std::min / std::max over the three vertices, first of equals)
__global__ void tri_boxes(const float* __restrict__ P, const uint32_t* __restrict__ I, uint32_t n, float4* bmin, float4* bmax,
                          float4* cen, uint32_t* order) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float* a = P + 3ull * I[3ull * t];
  const float* b = P + 3ull * I[3ull * t + 1];
  const float* c = P + 3ull * I[3ull * t + 2];
  float lo[3], hi[3], ce[3];
  for (int k = 0; k < 3; k++) {
    float l = b[k] < a[k] ? b[k] : a[k];
    l = c[k] < l ? c[k] : l;
    float h = a[k] < b[k] ? b[k] : a[k];
    h = h < c[k] ? c[k] : h;
    lo[k] = l; hi[k] = h;
    ce[k] = float(0.5 * (double(l) + double(h)));
  }
  bmin[t] = make_float4(lo[0], lo[1], lo[2], 0.0f);
  bmax[t] = make_float4(hi[0], hi[1], hi[2], 0.0f);
  cen[t] = make_float4(ce[0], ce[1], ce[2], 0.0f);
  order[t] = t;
}

inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

}  // namespace

// Builds the static BVH of (P, I) on the current device. False, with out untouched, when the root itself is a
// leaf (a handful of triangles: the host builder's special root) or on a CUDA error (err says which).
bool gpu_sah_build(const float* P, uint32_t n_verts, const uint32_t* I, uint32_t n, uint32_t leaf, vt::Bvh& out, std::string& err) {
  if (n < 2) return false;
  leaf = std::max(1u, leaf);
  const size_t nn = n;
  // one allocation: inputs, per-triangle records, order/scratch/qpos, shapes, two task lists x 2 levels, counters
  const size_t b_P = 3ull * n_verts * 4, b_I = 3ull * nn * 4, b_f4 = nn * 16, b_u = nn * 4, b_sh = nn * sizeof(Shape), b_t = nn * sizeof(Task);
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t total = al(b_P) + al(b_I) + 3 * al(b_f4) + 3 * al(b_u) + al(b_sh) + 4 * al(b_t) + 256;
  char* mem = nullptr;
  cudaStream_t st = nullptr;
  auto fail = [&](const char* what) {
    err = std::string("gpu bvh build: ") + what + ": " + cudaGetErrorString(cudaGetLastError());
    if (mem) cudaFree(mem);
    if (st) cudaStreamDestroy(st);
    return false;
  };
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return fail("stream");
  if (cudaMalloc(&mem, total) != cudaSuccess) return fail("allocation");
  size_t o = 0;
  auto take = [&](size_t b) { char* p = mem + o; o += al(b); return p; };
  float* dP = reinterpret_cast<float*>(take(b_P));
  uint32_t* dI = reinterpret_cast<uint32_t*>(take(b_I));
  Build B;
  float4* bmin = reinterpret_cast<float4*>(take(b_f4));
  float4* bmax = reinterpret_cast<float4*>(take(b_f4));
  float4* cen = reinterpret_cast<float4*>(take(b_f4));
  B.bmin = bmin; B.bmax = bmax; B.cen = cen;
  B.order = reinterpret_cast<uint32_t*>(take(b_u));
  B.scratch = reinterpret_cast<uint32_t*>(take(b_u));
  B.qpos = reinterpret_cast<int32_t*>(take(b_u));
  B.shapes = reinterpret_cast<Shape*>(take(b_sh));
  Task* lists[2][2];
  for (auto& l : lists) { l[0] = reinterpret_cast<Task*>(take(b_t)); l[1] = reinterpret_cast<Task*>(take(b_t)); }
  char* tail = mem + o;
  B.counters = reinterpret_cast<uint32_t*>(tail);          // 3 words
  B.root_box = reinterpret_cast<float*>(tail + 16);        // 6 floats
  B.root_leaf = reinterpret_cast<int32_t*>(tail + 48);
  B.leaf = leaf;
  if (cudaMemcpyAsync(dP, P, b_P, cudaMemcpyHostToDevice, st) != cudaSuccess || cudaMemcpyAsync(dI, I, b_I, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return fail("upload");
  cudaMemsetAsync(tail, 0, 64, st);
  tri_boxes<<<(n + 255) / 256, 256, 0, st>>>(dP, dI, n, bmin, bmax, cen, B.order);
  const Task root{0, int32_t(n), -1, 0};
  uint32_t nb = n >= uint32_t(BIG_TASK) ? 1 : 0, ns = 1 - nb;
  if (cudaMemcpyAsync(lists[0][nb ? 0 : 1], &root, sizeof(Task), cudaMemcpyHostToDevice, st) != cudaSuccess) return fail("upload");
  int cur = 0;
  uint32_t counts[3];
  for (int level = 0; nb + ns > 0; level++) {
    if (level > 4096) return fail("level cap");
    B.next_big = lists[cur ^ 1][0];
    B.next_small = lists[cur ^ 1][1];
    cudaMemsetAsync(B.counters + 1, 0, 8, st);
    if (nb) big_tasks<<<nb, BT, 0, st>>>(B, lists[cur][0]);
    if (ns) small_tasks<<<(ns + WPB - 1) / WPB, 32 * WPB, 0, st>>>(B, lists[cur][1], ns);
    if (cudaMemcpyAsync(counts, B.counters, 12, cudaMemcpyDeviceToHost, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
      return fail("level");
    nb = counts[1];
    ns = counts[2];
    cur ^= 1;
  }
  int32_t root_leaf = 0;
  float root_box[6];
  cudaMemcpyAsync(&root_leaf, B.root_leaf, 4, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(root_box, B.root_box, 24, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail("readback");
  if (root_leaf) { cudaFree(mem); cudaStreamDestroy(st); return false; }
  const uint32_t n_shapes = counts[0];
  std::vector<Shape> shapes(n_shapes);
  vt::Bvh bv;
  bv.order.resize(n);
  cudaMemcpyAsync(shapes.data(), B.shapes, size_t(n_shapes) * sizeof(Shape), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(bv.order.data(), B.order, b_u, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail("readback");
  cudaFree(mem);
  cudaStreamDestroy(st);
  // node numbers in the host builder's task order: pop a node, number its interior children (slot 0 then 1), push them
  struct Item { int32_t shape; uint32_t node, depth; };
  std::vector<Item> stack{{0, 0, 1}};
  bv.words.assign(VT_NODE_WORDS, 0u);
  bv.node_count = 1;
  bv.max_depth = 1;
  while (!stack.empty()) {
    const Item it = stack.back();
    stack.pop_back();
    bv.max_depth = std::max(bv.max_depth, it.depth);
    const Shape& S = shapes[it.shape];
    const int32_t lo[2] = {S.s, S.m}, hi[2] = {S.m, S.e};
    for (int slot = 0; slot < 2; slot++) {
      uint32_t ref, count;
      if (S.child[slot] < 0) {
        ref = uint32_t(lo[slot]); count = uint32_t(hi[slot] - lo[slot]);
      } else {
        ref = bv.node_count++;
        bv.words.resize(bv.words.size() + VT_NODE_WORDS, 0u);
        count = 0;
        stack.push_back({S.child[slot], ref, it.depth + 1});
      }
      uint32_t* w = bv.words.data() + size_t(it.node) * VT_NODE_WORDS + slot * 8;
      w[0] = fbits(S.lo[slot][0]); w[1] = fbits(S.lo[slot][1]); w[2] = fbits(S.lo[slot][2]); w[3] = ref;
      w[4] = fbits(S.hi[slot][0]); w[5] = fbits(S.hi[slot][1]); w[6] = fbits(S.hi[slot][2]); w[7] = count;
    }
  }
  for (int k = 0; k < 3; k++) { bv.lo[k] = root_box[k]; bv.hi[k] = root_box[3 + k]; }
  out = std::move(bv);
  return true;
}

}  // namespace vtk
