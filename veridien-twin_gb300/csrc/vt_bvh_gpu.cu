// Binned-SAH BVH2 build on the GPU: the tree of vt::sah_build (gpu/bvh.js:18-161), word for word.
//
// The host builder decides each node from its slot range alone. It computes the range's bounds, bins the
// centroids in 16 bins per axis, takes the cheapest SAH split (traversal and intersection cost 1), and partitions
// the slot order in place with gpu/bvh.js's swap-with-the-end loop. The nodes are then numbered in LIFO task
// order. Here every level of the tree is one pass over its tasks. A task of at least BIG_TASK slots is spread over
// blocks of CHUNK slots (six launches per level); one of at least MID_TASK slots gets a block, one of more than TINY
// slots a warp, a smaller one a thread. A task computes bounds, bins, SAH
// choice and partition, then appends its two children to the next level. Two passes per level over the decided
// shapes (subtree sizes up, numbers down) give the LIFO numbering and write the node words, so the node array is
// the host builder's.
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
#include <cstdio>
#include <cstdlib>
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
#ifndef VT_BVH_CHUNK
#define VT_BVH_CHUNK 4096
#endif
constexpr int BT = VT_BVH_BLOCK;   // threads of a big task's block
constexpr int BIG_TASK = VT_BVH_BIG;   // ranges of at least this many slots are big tasks
constexpr int CHUNK = VT_BVH_CHUNK;    // slots of a big task per block
constexpr int TINY = 32;               // ranges of at most this many slots are decided by one thread
#ifndef VT_BVH_MID
#define VT_BVH_MID 1024
#endif
constexpr int MID_TASK = VT_BVH_MID;   // ranges of at least this many slots (and below BIG_TASK) get a block
constexpr int MT = 256;                // threads of a mid task's block
constexpr int WPB = 8;             // warp tasks per 256-thread block
constexpr int THR_MIN = 64;        // ranges above this many slots bin through float thresholds

struct Task { int32_t s, e, parent, slot; };
struct Shape { int32_t s, e, m, child[2]; float lo[2][3], hi[2][3]; };

struct Build {
  const float4 *bmin, *bmax, *cen;   // per triangle: box and centroid (xyz)
  uint32_t *order, *scratch;
  int32_t* qpos;
  Shape* shapes;
  uint32_t* counters;                // [0] shapes, next [1] big, [2] small, [3] tiny and [4] mid tasks
  Task *next_big, *next_small, *next_tiny, *next_mid;
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

// Bounds of the slots [a, b) of the task that starts at s: node-box keys (value, then the slot's offset from s, so
// that the first slot among equal values wins) and the plain centroid box, reduced over the group.
template <int G>
__device__ __forceinline__ void range_bounds(const Build& B, int32_t s, int32_t a, int32_t b, const Grp<G>& g, unsigned long long* klo,
                                             unsigned long long* khi, float* clo, float* chi) {
  for (int k = 0; k < 3; k++) { klo[k] = ~0ull; khi[k] = 0ull; clo[k] = INFINITY; chi[k] = -INFINITY; }
  for (int32_t p = a + g.lane; p < b; p += G) {
    const uint32_t t = B.order[p];
    const float4 lo = B.bmin[t], hi = B.bmax[t], c = B.cen[t];
    const uint32_t off = uint32_t(p - s);
    for (int k = 0; k < 3; k++) {
      const float av = comp(lo, k), zv = comp(hi, k);
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
}

// the node box from the reduced keys: the values of the slots they name
__device__ __forceinline__ void key_box(const Build& B, int32_t s, const unsigned long long* klo, const unsigned long long* khi, float* lo, float* hi) {
  for (int k = 0; k < 3; k++) {
    lo[k] = comp(B.bmin[B.order[s + uint32_t(klo[k] & 0xffffffffu)]], k);
    hi[k] = comp(B.bmax[B.order[s + (0xffffffffu - uint32_t(khi[k] & 0xffffffffu))]], k);
  }
}

__device__ __forceinline__ void write_box(const Build& B, const Task& T, const float* lo, const float* hi) {
  if (T.parent >= 0) {
    Shape& P = B.shapes[T.parent];
    for (int k = 0; k < 3; k++) { P.lo[T.slot][k] = lo[k]; P.hi[T.slot][k] = hi[k]; }
  } else {
    for (int k = 0; k < 3; k++) { B.root_box[k] = lo[k]; B.root_box[3 + k] = hi[k]; }
  }
}

// bins per axis with a positive centroid extent
__device__ __forceinline__ void bin_frame(const float* clo, const float* chi, double* origin, double* scale, bool* use) {
  for (int k = 0; k < 3; k++) {
    origin[k] = double(clo[k]);
    const double extent = double(chi[k]) - origin[k];
    use[k] = extent > 0;
    scale[k] = use[k] ? BINS / extent : 0.0;
  }
}

// empty bins and, for a range of more than THR_MIN slots, each axis' 15 float thresholds (FP64 is a small fraction
// of FP32 on this part: such a range bins its centroids through bin_threshold's floats instead of one double
// expression per slot and axis)
template <int G>
__device__ __forceinline__ void bins_clear(GroupSh& sh, const Grp<G>& g, bool thr, const double* origin, const double* scale, const bool* use) {
  for (int i = g.lane; i < 3 * BINS; i += G) {
    (&sh.cnt[0][0])[i] = 0;
    for (int k = 0; k < 3; k++) { (&sh.blo[0][0][0])[3 * i + k] = 0xffffffffu; (&sh.bhi[0][0][0])[3 * i + k] = 0u; }
    if (thr && i < 3 * (BINS - 1)) {
      const int ax = i / (BINS - 1), b = i % (BINS - 1) + 1;
      sh.thr[ax][b - 1] = use[ax] ? bin_threshold(origin[ax], scale[ax], b) : INFINITY;
    }
  }
}

// the slots [a, b) into the group's shared bins
template <int G>
__device__ __forceinline__ void bins_fill(const Build& B, GroupSh& sh, const Grp<G>& g, int32_t a, int32_t b, bool thr, const double* origin,
                                          const double* scale, const bool* use) {
  for (int32_t p = a + g.lane; p < b; p += G) {
    const uint32_t t = B.order[p];
    const float4 lo = B.bmin[t], hi = B.bmax[t], c = B.cen[t];
    for (int ax = 0; ax < 3; ax++) {
      if (!use[ax]) continue;
      const int bn = thr ? bin_by_threshold(sh.thr[ax], comp(c, ax)) : bin_of(comp(c, ax), origin[ax], scale[ax]);
      atomicAdd(&sh.cnt[ax][bn], 1u);
      for (int k = 0; k < 3; k++) {
        atomicMin(&sh.blo[ax][bn][k], ord(comp(lo, k)));
        atomicMax(&sh.bhi[ax][bn][k], ord(comp(hi, k)));
      }
    }
  }
}

// SAH choice (gpu/bvh.js:60-118) over the bins in shared memory, on the group's first warp: a 16-lane segment per
// axis holds its bins, prefix and suffix boxes come from segmented scans, and lane b prices the split after bin b.
// Only splits after a non-empty bin are priced: the splits that follow an empty bin cost exactly what the last split
// after a non-empty bin costs, and the host's strict comparison keeps the earlier one. The cheapest split wins, ties
// to the lower (axis, bin), which is the host's loop order. Leaves sh.dec = {axis, bin, split}, split -1 for a leaf,
// -2 for the median without partition, 0 for a partition at (axis, bin).
__device__ void choose_split(GroupSh& sh, int lane, const float* box_lo, const float* box_hi, const bool* use, int32_t cnt, uint32_t leaf) {
  if (lane >= 32) return;
  const int l16 = lane & 15;
  double plo[3], phi[3];
  for (int k = 0; k < 3; k++) { plo[k] = double(box_lo[k]); phi[k] = double(box_hi[k]); }
  const double parent = half_area(plo, phi);
  double best_cost = INFINITY;
  int best_idx = 1 << 30;
  for (int round = 0; round < 2; round++) {
    const int ax = round * 2 + (lane >> 4);
    const bool live = ax < 3 && use[ax < 3 ? ax : 0];
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
  if (lane == 0) {
    const int best_axis = best_idx < (1 << 30) ? best_idx >> 4 : -1, best_bin = best_axis >= 0 ? best_idx & 15 : -1;
    int split = 0;
    if (best_axis < 0) split = cnt > int32_t(leaf) * 4 ? -2 : -1;
    else if (cnt <= int32_t(leaf) && best_cost >= double(cnt)) split = -1;
    sh.dec[0] = best_axis; sh.dec[1] = best_bin; sh.dec[2] = split;
  }
}

// an interior node over [s, e) split at m: its shape, and its two children as tasks of the next level
__device__ void emit_node(const Build& B, const Task& T, int32_t m) {
  const uint32_t id = atomicAdd(B.counters, 1u);
  Shape& S = B.shapes[id];
  S.s = T.s; S.e = T.e; S.m = m; S.child[0] = -1; S.child[1] = -1;
  if (T.parent >= 0) B.shapes[T.parent].child[T.slot] = int32_t(id);
  auto push = [&](const Task c) {
    if (c.e - c.s >= BIG_TASK) B.next_big[atomicAdd(B.counters + 1, 1u)] = c;
    else if (c.e - c.s >= MID_TASK) B.next_mid[atomicAdd(B.counters + 4, 1u)] = c;
    else if (c.e - c.s > TINY) B.next_small[atomicAdd(B.counters + 2, 1u)] = c;
    else B.next_tiny[atomicAdd(B.counters + 3, 1u)] = c;
  };
  push(Task{T.s, m, int32_t(id), 0});
  push(Task{m, T.e, int32_t(id), 1});
}

// one task on one group: bounds, SAH choice, partition, children
template <int G>
__device__ void run_task(const Build& B, const Task T, const Grp<G>& g) {
  GroupSh& sh = *g.sh;
  const int32_t s = T.s, e = T.e, cnt = e - s;
  unsigned long long klo[3], khi[3];
  float clo[3], chi[3], lo[3], hi[3];
  range_bounds(B, s, s, e, g, klo, khi, clo, chi);
  key_box(B, s, klo, khi, lo, hi);
  if (g.lane == 0) write_box(B, T, lo, hi);
  if (cnt <= 1) {
    if (g.lane == 0 && T.parent < 0) *B.root_leaf = 1;
    return;
  }
  double origin[3], scale[3];
  bool use[3];
  bin_frame(clo, chi, origin, scale, use);
  const bool thr = cnt > THR_MIN;
  bins_clear(sh, g, thr, origin, scale, use);
  g.sync();
  bins_fill(B, sh, g, s, e, thr, origin, scale, use);
  g.sync();
  choose_split(sh, g.lane, lo, hi, use, cnt, B.leaf);
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
    const double o = origin[ax], sc = scale[ax];
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
  if (g.lane == 0) emit_node(B, T, m);
}

__global__ void __launch_bounds__(MT) mid_tasks(Build B, const Task* __restrict__ tasks) {
  __shared__ GroupSh sh;
  const Grp<MT> g{int(threadIdx.x), int(threadIdx.x >> 5), &sh};
  run_task<MT>(B, tasks[blockIdx.x], g);
}

__global__ void __launch_bounds__(32 * WPB) small_tasks(Build B, const Task* __restrict__ tasks, uint32_t n) {
  __shared__ GroupSh sh[WPB];
  const uint32_t w = threadIdx.x >> 5, i = blockIdx.x * WPB + w;
  if (i >= n) return;   // whole warps leave: a warp task synchronises only within its warp
  Grp<32> g{int(threadIdx.x & 31), 0, &sh[w]};
  run_task<32>(B, tasks[i], g);
}

// A range of at most TINY slots on one thread, in the host builder's own sequential form: node box by strict
// comparisons (the first slot among equal values), bins by the double expression, the SAH price of each split after
// a non-empty bin from the two sides' boxes, and gpu/bvh.js's swap-with-the-end partition.
//
// FP64 issues at a small fraction of FP32 on this part, so a lane visits only its own splits (the set bits of its
// bins), and splits are compared on the undivided sum X = n_l A_l + n_r A_r. The host's cost 1 + X / parent does
// not decrease with X, and it keeps the first split of least cost. Two sums more than tol = (parent + X) 2^-49
// apart (eight units in the last place of the cost) give different costs, so only splits within tol of the best
// sum get the exact cost and the host's strict comparison; a degenerate or non-finite parent area takes the exact
// cost of every split.
__device__ __forceinline__ double sah_cost(double X, double parent) { return 1.0 + 1.0 * X / parent; }

__global__ void __launch_bounds__(128) tiny_tasks(Build B, const Task* __restrict__ tasks, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Task T = tasks[i];
  const int32_t s = T.s, e = T.e, cnt = e - s;
  uint32_t tt[TINY];
  float lo[3], hi[3], clo[3], chi[3];
  for (int j = 0; j < cnt; j++) {
    const uint32_t t = B.order[s + j];
    tt[j] = t;
    const float4 a = B.bmin[t], z = B.bmax[t], c = B.cen[t];
    for (int k = 0; k < 3; k++) {
      if (j == 0 || comp(a, k) < lo[k]) lo[k] = comp(a, k);
      if (j == 0 || comp(z, k) > hi[k]) hi[k] = comp(z, k);
      clo[k] = j == 0 ? comp(c, k) : fminf(clo[k], comp(c, k));
      chi[k] = j == 0 ? comp(c, k) : fmaxf(chi[k], comp(c, k));
    }
  }
  write_box(B, T, lo, hi);
  if (cnt <= 1) {
    if (T.parent < 0) *B.root_leaf = 1;
    return;
  }
  double origin[3], scale[3];
  bool use[3];
  bin_frame(clo, chi, origin, scale, use);
  double plo[3], phi[3];
  for (int k = 0; k < 3; k++) { plo[k] = double(lo[k]); phi[k] = double(hi[k]); }
  const double parent = half_area(plo, phi);
  const bool exact = !(parent > 0.0 && parent < INFINITY);
  double best_x = 0.0, best_cost = INFINITY;   // best_cost NaN: not yet computed for best_x
  int best_axis = -1, best_bin = -1;
  uint8_t bn[TINY];
  for (int ax = 0; ax < 3; ax++) {
    if (!use[ax]) continue;
    uint32_t present = 0;
    for (int j = 0; j < cnt; j++) {
      bn[j] = uint8_t(bin_of(comp(B.cen[tt[j]], ax), origin[ax], scale[ax]));
      present |= 1u << bn[j];
    }
    // the splits after a non-empty bin with something to their right, in increasing bin order
    for (uint32_t cand = present & ((1u << (31 - __clz(present))) - 1u); cand; cand &= cand - 1u) {
      const int v = __ffs(cand) - 1;
      float ll[3] = {INFINITY, INFINITY, INFINITY}, lh[3] = {-INFINITY, -INFINITY, -INFINITY};
      float rl[3] = {INFINITY, INFINITY, INFINITY}, rh[3] = {-INFINITY, -INFINITY, -INFINITY};
      uint32_t nl = 0;
      for (int j = 0; j < cnt; j++) {
        const float4 a = B.bmin[tt[j]], z = B.bmax[tt[j]];
        const bool L = bn[j] <= v;
        nl += L ? 1u : 0u;
        float* xl = L ? ll : rl;
        float* xh = L ? lh : rh;
        for (int k = 0; k < 3; k++) { xl[k] = fminf(xl[k], comp(a, k)); xh[k] = fmaxf(xh[k], comp(z, k)); }
      }
      const double la[3] = {double(ll[0]), double(ll[1]), double(ll[2])}, lb[3] = {double(lh[0]), double(lh[1]), double(lh[2])};
      const double ra[3] = {double(rl[0]), double(rl[1]), double(rl[2])}, rb[3] = {double(rh[0]), double(rh[1]), double(rh[2])};
      const double X = double(nl) * half_area(la, lb) + double(uint32_t(cnt) - nl) * half_area(ra, rb);
      bool take;
      if (exact || best_axis < 0) {
        const double c = sah_cost(X, parent);
        if (best_axis >= 0 && best_cost != best_cost) best_cost = sah_cost(best_x, parent);
        take = c < best_cost;
        if (take) best_cost = c;
      } else {
        const double tol = (parent + best_x) * 0x1p-49;
        if (X < best_x - tol) {
          take = true;
          best_cost = NAN;
        } else if (X > best_x + tol) {
          take = false;
        } else {
          if (best_cost != best_cost) best_cost = sah_cost(best_x, parent);
          const double c = sah_cost(X, parent);
          take = c < best_cost;
          if (take) best_cost = c;
        }
      }
      if (take) { best_x = X; best_axis = ax; best_bin = v; }
    }
  }
  if (best_axis >= 0 && best_cost != best_cost) best_cost = sah_cost(best_x, parent);
  int32_t m;
  if (best_axis < 0) {
    if (cnt <= int32_t(B.leaf) * 4) {
      if (T.parent < 0) *B.root_leaf = 1;
      return;
    }
    m = s + (cnt >> 1);
  } else if (cnt <= int32_t(B.leaf) && best_cost >= double(cnt)) {
    if (T.parent < 0) *B.root_leaf = 1;
    return;
  } else {
    int32_t a = 0, b = cnt - 1;
    while (a <= b) {
      const uint32_t t = tt[a];
      if (bin_of(comp(B.cen[t], best_axis), origin[best_axis], scale[best_axis]) <= best_bin) a++;
      else { tt[a] = tt[b]; tt[b] = t; b--; }
    }
    for (int j = 0; j < cnt; j++) B.order[s + j] = tt[j];
    const int32_t m0 = s + a;
    m = (m0 == s || m0 == e) ? s + (cnt >> 1) : m0;
  }
  emit_node(B, T, m);
}

// A task of at least BIG_TASK slots is spread over blocks of CHUNK slots each, in six launches per tree level:
// bounds (per-chunk partial keys), bins (each block reduces the partials, bins its chunk in shared memory and merges
// into the task's bins in global memory), choice and left counts (every block of the task prices the same bins), the
// partition's two passes, and the copy back with the node's children. The partition is the same closed form: a
// chunk's ranks among the left slots of [m0, e) counted from the top, and among the right slots of [s, m0) counted
// from the bottom, start after the chunks above it (all of them in [m0, e)) and below it (all in [s, m0)), so only
// the per-chunk left counts cross blocks.
struct BigState {
  float lo[3], hi[3];                // node box
  double origin[3], scale[3];
  int32_t use[3];
  float thr[3][BINS - 1];
  uint32_t cnt[3][BINS];
  uint32_t blo[3][BINS][3], bhi[3][BINS][3];
  int32_t axis, bin, split, m0, K;
};

struct Big {
  const Task* tasks;                 // this level's big tasks
  const uint32_t* map;               // per block: its task
  const int32_t* info;               // per task: first block, number of chunks
  BigState* state;                   // per task
  unsigned long long* pk;            // per block: klo[3], khi[3]
  float* pc;                         // per block: clo[3], chi[3]
  uint32_t* nleft;                   // per block: left slots of its chunk
};

struct Chunk {
  Task T;
  uint32_t task;
  int32_t first, n, c, a, b;         // first block and number of chunks of the task; this chunk and its slots [a, b)
};

__device__ __forceinline__ Chunk chunk_of(const Big& G, uint32_t blk) {
  Chunk C;
  C.task = G.map[blk];
  C.T = G.tasks[C.task];
  C.first = G.info[2 * C.task];
  C.n = G.info[2 * C.task + 1];
  C.c = int32_t(blk) - C.first;
  C.a = C.T.s + C.c * CHUNK;
  C.b = min(C.T.e, C.a + CHUNK);
  return C;
}

__global__ void __launch_bounds__(BT) big_bounds(Build B, Big G) {
  __shared__ GroupSh sh;
  const Grp<BT> g{int(threadIdx.x), int(threadIdx.x >> 5), &sh};
  const Chunk C = chunk_of(G, blockIdx.x);
  unsigned long long klo[3], khi[3];
  float clo[3], chi[3];
  range_bounds(B, C.T.s, C.a, C.b, g, klo, khi, clo, chi);
  if (g.lane == 0)
    for (int k = 0; k < 3; k++) {
      G.pk[6ull * blockIdx.x + k] = klo[k]; G.pk[6ull * blockIdx.x + 3 + k] = khi[k];
      G.pc[6ull * blockIdx.x + k] = clo[k]; G.pc[6ull * blockIdx.x + 3 + k] = chi[k];
    }
  if (C.c == 0) {
    BigState& S = G.state[C.task];
    for (int i = g.lane; i < 3 * BINS; i += BT) {
      (&S.cnt[0][0])[i] = 0u;
      for (int k = 0; k < 3; k++) { (&S.blo[0][0][0])[3 * i + k] = 0xffffffffu; (&S.bhi[0][0][0])[3 * i + k] = 0u; }
    }
  }
}

__global__ void __launch_bounds__(BT) big_bins(Build B, Big G) {
  __shared__ GroupSh sh;
  const Grp<BT> g{int(threadIdx.x), int(threadIdx.x >> 5), &sh};
  const Chunk C = chunk_of(G, blockIdx.x);
  BigState& S = G.state[C.task];
  unsigned long long klo[3], khi[3];
  float clo[3], chi[3];
  for (int k = 0; k < 3; k++) { klo[k] = ~0ull; khi[k] = 0ull; clo[k] = INFINITY; chi[k] = -INFINITY; }
  for (int j = g.lane; j < C.n; j += BT) {
    const size_t q = size_t(C.first + j);
    for (int k = 0; k < 3; k++) {
      klo[k] = min(klo[k], G.pk[6 * q + k]); khi[k] = max(khi[k], G.pk[6 * q + 3 + k]);
      clo[k] = fminf(clo[k], G.pc[6 * q + k]); chi[k] = fmaxf(chi[k], G.pc[6 * q + 3 + k]);
    }
  }
  for (int k = 0; k < 3; k++) {
    klo[k] = g.min64(klo[k]); khi[k] = g.max64(khi[k]);
    clo[k] = g.minf(clo[k]); chi[k] = g.maxf(chi[k]);
  }
  double origin[3], scale[3];
  bool use[3];
  bin_frame(clo, chi, origin, scale, use);
  bins_clear(sh, g, true, origin, scale, use);
  if (C.c == 0 && g.lane == 0) {
    float lo[3], hi[3];
    key_box(B, C.T.s, klo, khi, lo, hi);
    write_box(B, C.T, lo, hi);
    for (int k = 0; k < 3; k++) {
      S.lo[k] = lo[k]; S.hi[k] = hi[k];
      S.origin[k] = origin[k]; S.scale[k] = scale[k]; S.use[k] = use[k];
    }
  }
  g.sync();
  if (C.c == 0)
    for (int i = g.lane; i < 3 * (BINS - 1); i += BT) (&S.thr[0][0])[i] = (&sh.thr[0][0])[i];
  bins_fill(B, sh, g, C.a, C.b, true, origin, scale, use);
  g.sync();
  for (int i = g.lane; i < 3 * BINS; i += BT) {
    const uint32_t c = (&sh.cnt[0][0])[i];
    if (!c) continue;
    atomicAdd(&S.cnt[0][0] + i, c);
    for (int k = 0; k < 3; k++) {
      atomicMin(&S.blo[0][0][0] + 3 * i + k, (&sh.blo[0][0][0])[3 * i + k]);
      atomicMax(&S.bhi[0][0][0] + 3 * i + k, (&sh.bhi[0][0][0])[3 * i + k]);
    }
  }
}

// left of the split at (axis, bin): the centroid below the threshold of bin + 1
__device__ __forceinline__ bool big_left(const Build& B, int ax, float cut, uint32_t t) { return comp(B.cen[t], ax) < cut; }

__global__ void __launch_bounds__(BT) big_choose(Build B, Big G) {
  __shared__ GroupSh sh;
  const Grp<BT> g{int(threadIdx.x), int(threadIdx.x >> 5), &sh};
  const Chunk C = chunk_of(G, blockIdx.x);
  BigState& S = G.state[C.task];
  for (int i = g.lane; i < 3 * BINS; i += BT) {
    (&sh.cnt[0][0])[i] = (&S.cnt[0][0])[i];
    for (int k = 0; k < 3; k++) {
      (&sh.blo[0][0][0])[3 * i + k] = (&S.blo[0][0][0])[3 * i + k];
      (&sh.bhi[0][0][0])[3 * i + k] = (&S.bhi[0][0][0])[3 * i + k];
    }
  }
  g.sync();
  const float lo[3] = {S.lo[0], S.lo[1], S.lo[2]}, hi[3] = {S.hi[0], S.hi[1], S.hi[2]};
  const bool use[3] = {S.use[0] != 0, S.use[1] != 0, S.use[2] != 0};
  choose_split(sh, g.lane, lo, hi, use, C.T.e - C.T.s, B.leaf);
  g.sync();
  const int ax = sh.dec[0], bb = sh.dec[1], split = sh.dec[2];
  if (C.c == 0 && g.lane == 0) { S.axis = ax; S.bin = bb; S.split = split; }
  if (split != 0) return;
  const float cut = S.thr[ax][bb];
  uint32_t nl = 0;
  for (int32_t p = C.a + g.lane; p < C.b; p += BT) nl += big_left(B, ax, cut, B.order[p]) ? 1u : 0u;
  nl = g.sum(nl);
  if (g.lane == 0) G.nleft[blockIdx.x] = nl;
}

// m0 of the chunk's task, the left slots in the chunks above this one and the right slots in the chunks below it
__device__ __forceinline__ void big_offsets(const Big& G, const Chunk& C, const Grp<BT>& g, int32_t& m0, uint32_t& above, uint32_t& below) {
  uint32_t nl = 0, ab = 0, be = 0;
  for (int j = g.lane; j < C.n; j += BT) {
    const uint32_t L = G.nleft[C.first + j];
    nl += L;
    if (j > C.c) ab += L;
    if (j < C.c) be += uint32_t(min(C.T.e, C.T.s + (j + 1) * CHUNK) - (C.T.s + j * CHUNK)) - L;
  }
  m0 = C.T.s + int32_t(g.sum(nl));
  above = g.sum(ab);
  below = g.sum(be);
}

// pass 1: [m0, e) from the top (qpos of the left slots, right slots down one)
__global__ void __launch_bounds__(BT) big_part_top(Build B, Big G) {
  __shared__ GroupSh sh;
  const Grp<BT> g{int(threadIdx.x), int(threadIdx.x >> 5), &sh};
  const Chunk C = chunk_of(G, blockIdx.x);
  BigState& S = G.state[C.task];
  if (S.split != 0) return;
  int32_t m0;
  uint32_t above, below;
  big_offsets(G, C, g, m0, above, below);
  if (C.c == 0 && g.lane == 0) S.m0 = m0;
  const int ax = S.axis;
  const float cut = S.thr[ax][S.bin];
  const int32_t s = C.T.s, lo = max(C.a, m0);
  uint32_t K = above;
  for (int32_t base = 0; base < C.b - lo; base += BT) {
    const int32_t x = C.b - 1 - (base + g.lane);
    const bool valid = x >= lo;
    const uint32_t t = valid ? B.order[x] : 0u;
    const bool L = valid && big_left(B, ax, cut, t);
    uint32_t tot;
    const uint32_t r = g.scan(L, tot);
    if (L) B.qpos[s + K + r] = x;
    else if (valid && x > m0) B.scratch[x - 1] = t;
    K += tot;
  }
  if (g.lane == 0 && C.a <= m0 && m0 < C.b) S.K = int32_t(K);
}

// pass 2: [s, m0) from the bottom, and the slot at m0
__global__ void __launch_bounds__(BT) big_part_bottom(Build B, Big G) {
  __shared__ GroupSh sh;
  const Grp<BT> g{int(threadIdx.x), int(threadIdx.x >> 5), &sh};
  const Chunk C = chunk_of(G, blockIdx.x);
  const BigState& S = G.state[C.task];
  if (S.split != 0) return;
  int32_t m0;
  uint32_t above, below;
  big_offsets(G, C, g, m0, above, below);
  const int ax = S.axis;
  const float cut = S.thr[ax][S.bin];
  const int32_t s = C.T.s, e = C.T.e, hi = min(C.b, m0);
  if (g.lane == 0 && C.a <= m0 && m0 < C.b) {
    const uint32_t t = B.order[m0];
    const int32_t K = S.K;
    if (!big_left(B, ax, cut, t)) B.scratch[(K ? B.qpos[s + K - 1] : e) - 1] = t;
  }
  uint32_t k0 = below;
  for (int32_t base = 0; base < hi - C.a; base += BT) {
    const int32_t p = C.a + base + g.lane;
    const bool valid = p < hi;
    const uint32_t t = valid ? B.order[p] : 0u;
    const bool R = valid && !big_left(B, ax, cut, t);
    uint32_t tot;
    const uint32_t r = g.scan(R, tot);
    if (R) {
      const uint32_t k = k0 + r + 1;
      B.scratch[(k == 1 ? e : B.qpos[s + k - 2]) - 1] = t;
      B.scratch[p] = B.order[B.qpos[s + k - 1]];
    } else if (valid) {
      B.scratch[p] = t;
    }
    k0 += tot;
  }
}

// the partitioned chunk back into the slot order; the task's first block records the node and its children
__global__ void __launch_bounds__(BT) big_finish(Build B, Big G) {
  const Chunk C = chunk_of(G, blockIdx.x);
  const BigState& S = G.state[C.task];
  const int32_t s = C.T.s, e = C.T.e, cnt = e - s;
  if (S.split == 0)
    for (int32_t p = C.a + int32_t(threadIdx.x); p < C.b; p += BT) B.order[p] = B.scratch[p];
  if (C.c != 0 || threadIdx.x != 0) return;
  if (S.split == -1) {
    if (C.T.parent < 0) *B.root_leaf = 1;
    return;
  }
  const int32_t m0 = S.m0;
  const int32_t m = (S.split == -2 || m0 == s || m0 == e) ? s + (cnt >> 1) : m0;
  emit_node(B, C.T, m);
}

// Node numbers in the host builder's task order (pop a node, number its interior children slot 0 then slot 1, push
// them), without the replay: a node popped at counter c numbers its children c, c + 1, and the slot-1 child's
// subtree is processed before the slot-0 child's. So the slot-1 child is popped at c + (interior children) and the
// slot-0 child after the slot-1 child's D interior descendants, where D sums 1 + D over a node's interior children.
// The shapes of one tree level are one contiguous id range (the level's emits finish before the next level starts),
// so D is one launch per level from the deepest up and the numbers one launch per level from the root down, which
// also writes each node's 16 words.
__global__ void number_up(const Shape* __restrict__ S, int32_t* D, uint32_t a, uint32_t b) {
  const uint32_t i = a + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b) return;
  int32_t d = 0;
  for (int slot = 0; slot < 2; slot++) {
    const int32_t c = S[i].child[slot];
    if (c >= 0) d += 1 + D[c];
  }
  D[i] = d;
}

__global__ void number_down(const Shape* __restrict__ S, const int32_t* __restrict__ D, int32_t* num, int32_t* pop, uint32_t a, uint32_t b,
                            uint32_t* words) {
  const uint32_t i = a + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b) return;
  const Shape X = S[i];
  int32_t k = pop[i];
  int32_t cn[2] = {-1, -1};
  for (int slot = 0; slot < 2; slot++)
    if (X.child[slot] >= 0) { cn[slot] = k++; num[X.child[slot]] = cn[slot]; }
  if (X.child[1] >= 0) pop[X.child[1]] = k;
  if (X.child[0] >= 0) pop[X.child[0]] = k + (X.child[1] >= 0 ? D[X.child[1]] : 0);
  const int32_t lo[2] = {X.s, X.m}, hi[2] = {X.m, X.e};
  uint4* w = reinterpret_cast<uint4*>(words + size_t(num[i]) * VT_NODE_WORDS);
  for (int slot = 0; slot < 2; slot++) {
    const uint32_t ref = X.child[slot] >= 0 ? uint32_t(cn[slot]) : uint32_t(lo[slot]);
    const uint32_t count = X.child[slot] >= 0 ? 0u : uint32_t(hi[slot] - lo[slot]);
    w[2 * slot] = make_uint4(__float_as_uint(X.lo[slot][0]), __float_as_uint(X.lo[slot][1]), __float_as_uint(X.lo[slot][2]), ref);
    w[2 * slot + 1] = make_uint4(__float_as_uint(X.hi[slot][0]), __float_as_uint(X.hi[slot][1]), __float_as_uint(X.hi[slot][2]), count);
  }
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

}  // namespace

// Builds the static BVH of (P, I) on the current device. False, with out untouched, when the root itself is a
// leaf (a handful of triangles: the host builder's special root) or on a CUDA error (err says which).
bool gpu_sah_build(const float* P, uint32_t n_verts, const uint32_t* I, uint32_t n, uint32_t leaf, vt::Bvh& out, std::string& err) {
  if (n < 2) return false;
  leaf = std::max(1u, leaf);
  // VT_BVH_TIMING=1 prints the build's phases to stderr
  static const bool timing = [] { const char* v = std::getenv("VT_BVH_TIMING"); return v && *v && *v != '0'; }();
  using clk = std::chrono::steady_clock;
  const auto t_start = clk::now();
  auto ms = [&](clk::time_point a) { return std::chrono::duration<double, std::milli>(clk::now() - a).count(); };
  double ph[3] = {0, 0, 0};   // setup + upload, levels, numbering + readback
  auto mark = [&](int i, clk::time_point& a) { ph[i] = ms(a); a = clk::now(); };
  clk::time_point tp = t_start;
  int n_levels = 0;
  const size_t nn = n;
  // one allocation: inputs, per-triangle records, order/scratch/qpos, shapes, four task lists x 2 level parities, the
  // big tasks' chunk state, the numbering arrays and node words, counters
  const size_t b_P = 3ull * n_verts * 4, b_I = 3ull * nn * 4, b_f4 = nn * 16, b_u = nn * 4, b_sh = nn * sizeof(Shape), b_t = nn * sizeof(Task);
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  // big tasks of one level: at most n / BIG_TASK of them, in at most n / CHUNK + (tasks) chunks
  const size_t max_big = nn / BIG_TASK + 2, max_chunks = nn / CHUNK + max_big + 2;
  const size_t b_state = max_big * sizeof(BigState), b_pk = max_chunks * 48, b_pc = max_chunks * 24, b_nl = max_chunks * 4,
               b_map = (max_chunks + 2 * max_big) * 4;
  // numbering: D, number and pop counter per shape, 16 words per node
  const size_t b_num = nn * 4, b_words = nn * VT_NODE_WORDS * 4;
  const size_t total = al(b_P) + al(b_I) + 3 * al(b_f4) + 3 * al(b_u) + al(b_sh) + 8 * al(b_t) + al(b_state) + al(b_pk) + al(b_pc) + al(b_nl) +
                       al(b_map) + 3 * al(b_num) + al(b_words) + 256;
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
  Task* lists[2][4];   // per level parity: big, small, tiny and mid tasks
  for (auto& l : lists)
    for (auto& x : l) x = reinterpret_cast<Task*>(take(b_t));
  Big G;
  G.state = reinterpret_cast<BigState*>(take(b_state));
  G.pk = reinterpret_cast<unsigned long long*>(take(b_pk));
  G.pc = reinterpret_cast<float*>(take(b_pc));
  G.nleft = reinterpret_cast<uint32_t*>(take(b_nl));
  uint32_t* dmap = reinterpret_cast<uint32_t*>(take(b_map));
  int32_t* dD = reinterpret_cast<int32_t*>(take(b_num));
  int32_t* dnum = reinterpret_cast<int32_t*>(take(b_num));
  int32_t* dpop = reinterpret_cast<int32_t*>(take(b_num));
  uint32_t* dwords = reinterpret_cast<uint32_t*>(take(b_words));
  char* tail = mem + o;
  B.counters = reinterpret_cast<uint32_t*>(tail);          // 5 words
  B.root_box = reinterpret_cast<float*>(tail + 32);        // 6 floats
  B.root_leaf = reinterpret_cast<int32_t*>(tail + 64);
  B.leaf = leaf;
  if (cudaMemcpyAsync(dP, P, b_P, cudaMemcpyHostToDevice, st) != cudaSuccess || cudaMemcpyAsync(dI, I, b_I, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return fail("upload");
  cudaMemsetAsync(tail, 0, 128, st);
  tri_boxes<<<(n + 255) / 256, 256, 0, st>>>(dP, dI, n, bmin, bmax, cen, B.order);
  if (timing) { cudaStreamSynchronize(st); mark(0, tp); }
  const Task root{0, int32_t(n), -1, 0};
  uint32_t nb = n >= uint32_t(BIG_TASK) ? 1 : 0, nm = !nb && n >= uint32_t(MID_TASK) ? 1 : 0, nt = n <= uint32_t(TINY) ? 1 : 0,
           ns = 1 - nb - nm - nt;
  if (cudaMemcpyAsync(lists[0][nb ? 0 : nm ? 3 : nt ? 2 : 1], &root, sizeof(Task), cudaMemcpyHostToDevice, st) != cudaSuccess) return fail("upload");
  int cur = 0;
  uint32_t counts[5];
  std::vector<Task> big;              // this level's big tasks, read back after each level
  std::vector<uint32_t> plan;         // per block its task, then per task its first block and chunk count
  std::vector<uint32_t> level_end;    // shapes emitted up to and including each level
  if (nb) big.push_back(root);
  for (int level = 0; nb + nm + ns + nt > 0; level++) {
    if (level > 4096) return fail("level cap");
    B.next_big = lists[cur ^ 1][0];
    B.next_small = lists[cur ^ 1][1];
    B.next_tiny = lists[cur ^ 1][2];
    B.next_mid = lists[cur ^ 1][3];
    cudaMemsetAsync(B.counters + 1, 0, 16, st);
    if (nb) {
      uint32_t blocks = 0;
      for (const Task& t : big) blocks += uint32_t((t.e - t.s + CHUNK - 1) / CHUNK);
      if (blocks > max_chunks || nb > max_big) return fail("chunk plan");
      plan.assign(size_t(blocks) + 2 * nb, 0u);
      uint32_t first = 0;
      for (uint32_t i = 0; i < nb; i++) {
        const uint32_t k = uint32_t((big[i].e - big[i].s + CHUNK - 1) / CHUNK);
        for (uint32_t j = 0; j < k; j++) plan[first + j] = i;
        plan[blocks + 2 * i] = first;
        plan[blocks + 2 * i + 1] = k;
        first += k;
      }
      if (cudaMemcpyAsync(dmap, plan.data(), plan.size() * 4, cudaMemcpyHostToDevice, st) != cudaSuccess) return fail("chunk plan");
      G.tasks = lists[cur][0];
      G.map = dmap;
      G.info = reinterpret_cast<const int32_t*>(dmap + blocks);
      big_bounds<<<blocks, BT, 0, st>>>(B, G);
      big_bins<<<blocks, BT, 0, st>>>(B, G);
      big_choose<<<blocks, BT, 0, st>>>(B, G);
      big_part_top<<<blocks, BT, 0, st>>>(B, G);
      big_part_bottom<<<blocks, BT, 0, st>>>(B, G);
      big_finish<<<blocks, BT, 0, st>>>(B, G);
    }
    if (nm) mid_tasks<<<nm, MT, 0, st>>>(B, lists[cur][3]);
    if (ns) small_tasks<<<(ns + WPB - 1) / WPB, 32 * WPB, 0, st>>>(B, lists[cur][1], ns);
    if (nt) tiny_tasks<<<(nt + 127) / 128, 128, 0, st>>>(B, lists[cur][2], nt);
    if (cudaMemcpyAsync(counts, B.counters, 20, cudaMemcpyDeviceToHost, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
      return fail("level");
    nb = counts[1];
    ns = counts[2];
    nt = counts[3];
    nm = counts[4];
    level_end.push_back(counts[0]);
    big.resize(nb);
    if (nb && (cudaMemcpyAsync(big.data(), lists[cur ^ 1][0], nb * sizeof(Task), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
               cudaStreamSynchronize(st) != cudaSuccess))
      return fail("level");
    cur ^= 1;
    n_levels = level + 1;
  }
  if (timing) mark(1, tp);
  int32_t root_leaf = 0;
  float root_box[6];
  cudaMemcpyAsync(&root_leaf, B.root_leaf, 4, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(root_box, B.root_box, 24, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail("readback");
  if (root_leaf) { cudaFree(mem); cudaStreamDestroy(st); return false; }
  const uint32_t n_shapes = counts[0];
  // node numbers and words on the device; the tree's depth is the number of levels that emitted nodes
  vt::Bvh bv;
  uint32_t depth = 0;
  for (size_t L = 0; L < level_end.size(); L++)
    if (level_end[L] > (L ? level_end[L - 1] : 0u)) depth = uint32_t(L) + 1;
  for (size_t L = level_end.size(); L-- > 0;) {
    const uint32_t a = L ? level_end[L - 1] : 0u, b = level_end[L];
    if (b > a) number_up<<<(b - a + 255) / 256, 256, 0, st>>>(B.shapes, dD, a, b);
  }
  const int32_t root_init[2] = {0, 1};   // the root is node 0, popped at counter 1
  cudaMemcpyAsync(dnum, &root_init[0], 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dpop, &root_init[1], 4, cudaMemcpyHostToDevice, st);
  for (size_t L = 0; L < level_end.size(); L++) {
    const uint32_t a = L ? level_end[L - 1] : 0u, b = level_end[L];
    if (b > a) number_down<<<(b - a + 255) / 256, 256, 0, st>>>(B.shapes, dD, dnum, dpop, a, b, dwords);
  }
  bv.words.resize(size_t(n_shapes) * VT_NODE_WORDS);
  bv.order.resize(n);
  bv.node_count = n_shapes;
  bv.max_depth = std::max(1u, depth);
  cudaMemcpyAsync(bv.words.data(), dwords, bv.words.size() * 4, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(bv.order.data(), B.order, b_u, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail("readback");
  cudaFree(mem);
  cudaStreamDestroy(st);
  if (timing) mark(2, tp);
  for (int k = 0; k < 3; k++) { bv.lo[k] = root_box[k]; bv.hi[k] = root_box[3 + k]; }
  out = std::move(bv);
  if (timing)
    std::fprintf(stderr, "gpu bvh build of %u triangles: %.2f ms (setup + upload %.2f, %d levels %.2f, numbering + readback %.2f)\n", n,
                 ms(t_start), ph[0], n_levels, ph[1], ph[2]);
  return true;
}

}  // namespace vtk
