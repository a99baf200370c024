// Scene preparation on a CUDA device: gpu/scene_gpu.js:68 weld and :95 subdivide with the numbering and arithmetic of
// the JavaScript (and of the host restatement, vt_scene_prep.cpp), bit for bit.
//
// Both number things in the order they are first met: weld a distinct (position, normal) key at its first vertex,
// subdivide an edge's midpoint at the first midpoint() call on that edge. On the device every occurrence carries its
// key and its position in input order; a sort by (key, position) gathers a key's occurrences in runs whose lead is
// the first one; the leads flagged in input order and scanned give the ids. The rest is per element: remapping,
// dropping degenerate triangles (with an order-keeping compaction), midpoints, re-triangulation. The arithmetic is in
// doubles without multiply-add contraction (this file is compiled with --fmad=false), as the host code does it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "vt_scene_prep.h"

namespace {

// ------------------------------------------------------------------------------------------------ device memory
// one-time load path: plain allocations, released on every return
struct DevBuf {
  void* p = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { if (p) cudaFree(p); }
  bool alloc(size_t bytes) {
    if (p) { cudaFree(p); p = nullptr; }
    if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) { cudaGetLastError(); p = nullptr; return false; }
    return true;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// ------------------------------------------------------------------------------------------------ sort
// (key, position) pairs, all distinct (positions are): a bitonic sort needs no stability
struct SortItem {
  unsigned long long k;
  uint32_t p, pad;
};
__device__ __forceinline__ bool item_less(const SortItem& a, const SortItem& b) { return a.k < b.k || (a.k == b.k && a.p < b.p); }

constexpr uint32_t CH = 2048;   // elements a block sorts in shared memory (1024 threads, one pair each)

// one compare-exchange step of distance j within bitonic sequences of size k, over the whole array
__global__ void bitonic_global(SortItem* a, uint32_t n, uint32_t k, uint32_t j) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t l = i ^ j;
  if (l <= i) return;
  const bool up = (i & k) == 0u;
  const SortItem x = a[i], y = a[l];
  if (up ? item_less(y, x) : item_less(x, y)) { a[i] = y; a[l] = x; }
}

// the steps j0, j0 / 2, ..., 1 of sequence size k on one CH-element chunk in shared memory
__global__ void __launch_bounds__(1024) bitonic_shared(SortItem* a, uint32_t k, uint32_t j0) {
  __shared__ SortItem s[CH];
  const uint32_t base = blockIdx.x * CH;
  for (uint32_t t = threadIdx.x; t < CH; t += blockDim.x) s[t] = a[base + t];
  __syncthreads();
  for (uint32_t j = j0; j > 0u; j >>= 1) {
    const uint32_t q = threadIdx.x;   // pair q of the chunk
    const uint32_t i = (q / j) * 2u * j + (q % j), l = i + j;
    const bool up = ((base + i) & k) == 0u;
    const SortItem x = s[i], y = s[l];
    if (up ? item_less(y, x) : item_less(x, y)) { s[i] = y; s[l] = x; }
    __syncthreads();
  }
  for (uint32_t t = threadIdx.x; t < CH; t += blockDim.x) a[base + t] = s[t];
}

// n: a power of two >= CH
void bitonic_sort(SortItem* a, uint32_t n, cudaStream_t st) {
  for (uint32_t k = 2; k <= n; k <<= 1) {
    uint32_t j = k >> 1;
    for (; j >= CH; j >>= 1) bitonic_global<<<n / 256, 256, 0, st>>>(a, n, k, j);
    bitonic_shared<<<n / CH, 1024, 0, st>>>(a, k, j);
  }
}

__global__ void fill_items(SortItem* a, uint32_t from, uint32_t n) {
  const uint32_t i = from + blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = SortItem{~0ull, ~0u, 0u};
}

uint32_t pow2_at_least(uint32_t n) {
  uint32_t p = CH;
  while (p < n) p <<= 1;
  return p;
}

// ------------------------------------------------------------------------------------------------ scan
// exclusive prefix sum of n words (in place allowed), the total into *total
constexpr uint32_t SB = 1024;
__global__ void __launch_bounds__(SB) scan_block(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* sums) {
  __shared__ uint32_t s[SB];
  const uint32_t i = blockIdx.x * SB + threadIdx.x;
  const uint32_t v = i < n ? in[i] : 0u;
  s[threadIdx.x] = v;
  __syncthreads();
  for (uint32_t o = 1; o < SB; o <<= 1) {
    const uint32_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - v;
  if (threadIdx.x == SB - 1) sums[blockIdx.x] = s[SB - 1];
}
__global__ void scan_add(uint32_t* out, uint32_t n, const uint32_t* offs) {
  const uint32_t i = blockIdx.x * SB + threadIdx.x;
  if (i < n) out[i] += offs[blockIdx.x];
}
__global__ void copy_word(const uint32_t* a, uint32_t* b) { *b = *a; }

bool scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, cudaStream_t st) {
  const uint32_t nb = (n + SB - 1) / SB;
  DevBuf sums, offs;
  if (!sums.alloc(size_t(nb + 1) * 4) || !offs.alloc(size_t(nb + 1) * 4)) return false;
  if (n) scan_block<<<nb, SB, 0, st>>>(in, out, n, sums.as<uint32_t>());
  if (nb <= 1) {
    if (n) copy_word<<<1, 1, 0, st>>>(sums.as<uint32_t>(), total);
    else cudaMemsetAsync(total, 0, 4, st);
  } else {
    if (!scan_exclusive(sums.as<uint32_t>(), offs.as<uint32_t>(), nb, total, st)) return false;
    scan_add<<<nb, SB, 0, st>>>(out, n, offs.as<uint32_t>());
  }
  // the block sums are released on return: their readers first
  if (cudaStreamSynchronize(st) != cudaSuccess) { cudaGetLastError(); return false; }
  return true;
}

// ------------------------------------------------------------------------------------------------ arithmetic
// JavaScript's Math.round: the nearest integer, halves toward +infinity
__device__ __forceinline__ long long js_round(double x) { return (long long)floor(x + 0.5); }

// Math.hypot of three numbers as V8 evaluates it: scaled by the largest magnitude, squares summed with Kahan
// compensation, square root times the scale
__device__ __forceinline__ double js_hypot3(double x, double y, double z) {
  const double v[3] = {fabs(x), fabs(y), fabs(z)};
  const double mx = fmax(v[0], fmax(v[1], v[2]));
  if (mx == 0) return 0;
  double sum = 0, comp = 0;
  for (int i = 0; i < 3; i++) {
    const double n = v[i] / mx;
    const double summand = n * n - comp;
    const double pre = sum + summand;
    comp = (pre - sum) - summand;
    sum = pre;
  }
  return sqrt(sum) * mx;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long h, unsigned long long v) {
  h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
  h ^= h >> 31;
  h *= 0xbf58476d1ce4e5b9ull;
  h ^= h >> 27;
  return h;
}

// ------------------------------------------------------------------------------------------------ weld
// per vertex: the six rounded key words (position x 1e7, normal x 1e4) and the item (hash of the key, vertex)
__global__ void weld_keys(const float* P, const float* N, uint32_t n, long long* key, SortItem* items) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  unsigned long long h = 0x243f6a8885a308d3ull;
  for (int c = 0; c < 3; c++) {
    const long long kp = js_round(double(P[3 * size_t(v) + c]) * 1e7), kn = js_round(double(N[3 * size_t(v) + c]) * 1e4);
    key[6 * size_t(v) + c] = kp;
    key[6 * size_t(v) + 3 + c] = kn;
  }
  for (int c = 0; c < 6; c++) h = mix64(h, (unsigned long long)key[6 * size_t(v) + c]);
  items[v] = SortItem{h, v, 0u};
}

__device__ __forceinline__ bool same_key(const long long* key, uint32_t a, uint32_t b) {
  for (int c = 0; c < 6; c++) if (key[6 * size_t(a) + c] != key[6 * size_t(b) + c]) return false;
  return true;
}

// per sorted item: the first vertex with the same key (the first of its hash run whose key matches; within a run the
// vertices are in increasing order); first[v] = 1 when v is that vertex
__global__ void weld_rep(const SortItem* items, uint32_t n, const long long* key, uint32_t* rep, uint32_t* first) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long h = items[i].k;
  const uint32_t v = items[i].p;
  uint32_t s = i;
  while (s > 0u && items[s - 1].k == h) s--;
  uint32_t r = v;
  for (uint32_t j = s; j < i; j++)
    if (same_key(key, items[j].p, v)) { r = items[j].p; break; }
  rep[v] = r;
  first[v] = r == v ? 1u : 0u;
}

// the welded vertices (at their ids) and every input vertex's id
__global__ void weld_out(const float* P, const float* N, uint32_t n, const uint32_t* rep, const uint32_t* id, double* P2, double* N2,
                         uint32_t* remap) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const uint32_t r = rep[v];
  remap[v] = id[r];
  if (r == v)
    for (int c = 0; c < 3; c++) { P2[3 * size_t(id[v]) + c] = double(P[3 * size_t(v) + c]); N2[3 * size_t(id[v]) + c] = double(N[3 * size_t(v) + c]); }
}

__global__ void weld_tri_keep(const uint32_t* I, uint32_t nt, const uint32_t* remap, uint32_t* keep) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const uint32_t a = remap[I[3 * size_t(t)]], b = remap[I[3 * size_t(t) + 1]], c = remap[I[3 * size_t(t) + 2]];
  keep[t] = (a == b || b == c || a == c) ? 0u : 1u;   // degenerate after welding
}
__global__ void weld_tri_out(const uint32_t* I, uint32_t nt, const uint32_t* remap, const uint32_t* keep, const uint32_t* at, uint32_t* I2) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt || !keep[t]) return;
  for (int c = 0; c < 3; c++) I2[3 * size_t(at[t]) + c] = remap[I[3 * size_t(t) + c]];
}

// ------------------------------------------------------------------------------------------------ subdivide
__device__ __forceinline__ double len2(const double* P, uint32_t a, uint32_t b) {
  const double x = P[3 * size_t(a)] - P[3 * size_t(b)], y = P[3 * size_t(a) + 1] - P[3 * size_t(b) + 1],
               z = P[3 * size_t(a) + 2] - P[3 * size_t(b) + 2];
  return x * x + y * y + z * z;
}
__device__ __forceinline__ unsigned long long edge_key(uint32_t a, uint32_t b) {
  return a < b ? ((unsigned long long)a << 32) | b : ((unsigned long long)b << 32) | a;
}

// a triangle's pattern of edges longer than h: the number split, and the edge the pattern starts from (the split edge
// for one, the unsplit edge for two)
struct Pattern { uint32_t v[3]; int cnt, e; };
__device__ __forceinline__ Pattern pattern(const double* P, const uint32_t* tris, uint32_t t, double h2) {
  Pattern q;
  for (int c = 0; c < 3; c++) q.v[c] = tris[3 * size_t(t) + c];
  const bool mk[3] = {len2(P, q.v[0], q.v[1]) > h2, len2(P, q.v[1], q.v[2]) > h2, len2(P, q.v[2], q.v[0]) > h2};
  q.cnt = int(mk[0]) + int(mk[1]) + int(mk[2]);
  q.e = q.cnt == 1 ? (mk[0] ? 0 : mk[1] ? 1 : 2) : q.cnt == 2 ? (!mk[0] ? 0 : !mk[1] ? 1 : 2) : 0;
  return q;
}

// per triangle: its midpoint() calls in the order the JavaScript makes them (slot 3 t + j), their edges, and how many
// triangles it becomes
__global__ void sub_calls(const double* P, const uint32_t* tris, uint32_t nt, double h2, SortItem* items, uint2* ends, uint32_t* out_cnt) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const Pattern q = pattern(P, tris, t, h2);
  uint2 e[3];
  int nc = 0;
  if (q.cnt == 3) {
    e[0] = make_uint2(q.v[0], q.v[1]); e[1] = make_uint2(q.v[1], q.v[2]); e[2] = make_uint2(q.v[2], q.v[0]);
    nc = 3;
  } else if (q.cnt == 1) {
    e[0] = make_uint2(q.v[q.e], q.v[(q.e + 1) % 3]);
    nc = 1;
  } else if (q.cnt == 2) {
    const uint32_t A = q.v[q.e], B = q.v[(q.e + 1) % 3], C = q.v[(q.e + 2) % 3];
    e[0] = make_uint2(B, C); e[1] = make_uint2(C, A);
    nc = 2;
  }
  for (int j = 0; j < 3; j++) {
    const uint32_t slot = 3 * t + j;
    items[slot] = j < nc ? SortItem{edge_key(e[j].x, e[j].y), slot, 0u} : SortItem{~0ull, slot, 0u};
    ends[slot] = j < nc ? e[j] : make_uint2(0u, 0u);
  }
  out_cnt[t] = uint32_t(q.cnt + 1);
}

// first[slot] = 1 for each edge's first call (the lead of its run in (edge, slot) order)
__global__ void sub_first(const SortItem* items, uint32_t n, uint32_t* first) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || items[i].k == ~0ull) return;
  first[items[i].p] = (i == 0u || items[i - 1].k != items[i].k) ? 1u : 0u;
}

// every call's vertex id (its run lead's), and at each lead the new vertex: the midpoint, the normalised mean normal
__global__ void sub_assign(const SortItem* items, uint32_t n, const uint32_t* rank, uint32_t n_v, const uint2* ends, double* P, double* N,
                           uint32_t* call_id) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long k = items[i].k;
  if (k == ~0ull) return;
  uint32_t s = i;
  while (s > 0u && items[s - 1].k == k) s--;
  const uint32_t lead = items[s].p;
  const uint32_t id = n_v + rank[lead];
  call_id[items[i].p] = id;
  if (s != i) return;
  const uint32_t a = ends[lead].x, b = ends[lead].y;
  for (int c = 0; c < 3; c++) P[3 * size_t(id) + c] = 0.5 * (P[3 * size_t(a) + c] + P[3 * size_t(b) + c]);
  double nx = N[3 * size_t(a)] + N[3 * size_t(b)], ny = N[3 * size_t(a) + 1] + N[3 * size_t(b) + 1], nz = N[3 * size_t(a) + 2] + N[3 * size_t(b) + 2];
  const double l = js_hypot3(nx, ny, nz);
  if (l > 1e-6) { nx /= l; ny /= l; nz /= l; } else { nx = N[3 * size_t(a)]; ny = N[3 * size_t(a) + 1]; nz = N[3 * size_t(a) + 2]; }
  N[3 * size_t(id)] = nx; N[3 * size_t(id) + 1] = ny; N[3 * size_t(id) + 2] = nz;
}

// each triangle's replacement at its offset, in the JavaScript's order; the pattern is evaluated on the positions
// of the pass's start (new vertices do not move old ones), the two-split case compares the quad's diagonals
__global__ void sub_emit(const double* P, const uint32_t* tris, uint32_t nt, double h2, const uint32_t* call_id, const uint32_t* at,
                         uint32_t* out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const Pattern q = pattern(P, tris, t, h2);
  uint32_t* o = out + 3 * size_t(at[t]);
  const uint32_t* m = call_id + 3 * size_t(t);
  if (q.cnt == 0) {
    o[0] = q.v[0]; o[1] = q.v[1]; o[2] = q.v[2];
  } else if (q.cnt == 3) {
    const uint32_t a = m[0], b = m[1], c = m[2];
    const uint32_t s[12] = {q.v[0], a, c, a, q.v[1], b, c, b, q.v[2], a, b, c};
    for (int k = 0; k < 12; k++) o[k] = s[k];
  } else if (q.cnt == 1) {
    const uint32_t p = q.v[q.e], qq = q.v[(q.e + 1) % 3], r = q.v[(q.e + 2) % 3], mm = m[0];
    const uint32_t s[6] = {p, mm, r, mm, qq, r};
    for (int k = 0; k < 6; k++) o[k] = s[k];
  } else {
    const uint32_t A = q.v[q.e], B = q.v[(q.e + 1) % 3], C = q.v[(q.e + 2) % 3], mBC = m[0], mCA = m[1];
    o[0] = mCA; o[1] = mBC; o[2] = C;
    if (len2(P, A, mBC) < len2(P, B, mCA)) { o[3] = A; o[4] = B; o[5] = mBC; o[6] = A; o[7] = mBC; o[8] = mCA; }
    else { o[3] = A; o[4] = B; o[5] = mCA; o[6] = B; o[7] = mBC; o[8] = mCA; }
  }
}

uint32_t grid_of(uint32_t n) { return std::max(1u, (n + 255) / 256); }

bool use_device(int32_t device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev || cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return true;
}

template <class T>
bool to_host(std::vector<T>& v, const void* d, size_t count) {
  v.resize(count);
  return !count || cudaMemcpy(v.data(), d, count * sizeof(T), cudaMemcpyDeviceToHost) == cudaSuccess;
}
uint32_t read_word(const uint32_t* d) {
  uint32_t v = 0;
  cudaMemcpy(&v, d, 4, cudaMemcpyDeviceToHost);
  return v;
}

}  // namespace

extern "C" {

vt_status vt_weld_device(int32_t device, const float* P, const float* N, uint32_t n_verts, const uint32_t* I, uint32_t n_idx, vt_mesh_out* out) {
  if (!out || (n_verts && (!P || !N)) || (n_idx && !I) || n_idx % 3) return VT_ERR_ARG;
  *out = vt_mesh_out{};
  for (uint32_t k = 0; k < n_idx; k++) if (I[k] >= n_verts) return VT_ERR_ARG;
  if (!use_device(device)) return VT_ERR_NO_DEVICE;
  cudaStream_t st = 0;
  const uint32_t nt = n_idx / 3, ns = pow2_at_least(std::max(n_verts, 1u));
  DevBuf dP, dN, dI, key, items, rep, first, id, tot, P2, N2, remap, keep, at, I2;
  if (!dP.alloc(size_t(n_verts) * 12) || !dN.alloc(size_t(n_verts) * 12) || !dI.alloc(size_t(n_idx) * 4) || !key.alloc(size_t(n_verts) * 48) ||
      !items.alloc(size_t(ns) * sizeof(SortItem)) || !rep.alloc(size_t(n_verts) * 4) || !first.alloc(size_t(n_verts) * 4) ||
      !id.alloc(size_t(n_verts) * 4) || !tot.alloc(16) || !P2.alloc(size_t(n_verts) * 24) || !N2.alloc(size_t(n_verts) * 24) ||
      !remap.alloc(size_t(n_verts) * 4) || !keep.alloc(size_t(nt) * 4) || !at.alloc(size_t(nt) * 4) || !I2.alloc(size_t(n_idx) * 4))
    return VT_ERR_OOM;
  if (cudaMemcpy(dP.p, P, size_t(n_verts) * 12, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dN.p, N, size_t(n_verts) * 12, cudaMemcpyHostToDevice) != cudaSuccess ||
      (n_idx && cudaMemcpy(dI.p, I, size_t(n_idx) * 4, cudaMemcpyHostToDevice) != cudaSuccess))
    return VT_ERR_CUDA;
  if (n_verts) weld_keys<<<grid_of(n_verts), 256, 0, st>>>(dP.as<float>(), dN.as<float>(), n_verts, key.as<long long>(), items.as<SortItem>());
  fill_items<<<grid_of(ns - n_verts), 256, 0, st>>>(items.as<SortItem>(), n_verts, ns);
  bitonic_sort(items.as<SortItem>(), ns, st);
  if (n_verts) weld_rep<<<grid_of(n_verts), 256, 0, st>>>(items.as<SortItem>(), n_verts, key.as<long long>(), rep.as<uint32_t>(), first.as<uint32_t>());
  if (!scan_exclusive(first.as<uint32_t>(), id.as<uint32_t>(), n_verts, tot.as<uint32_t>(), st)) return VT_ERR_CUDA;
  if (n_verts)
    weld_out<<<grid_of(n_verts), 256, 0, st>>>(dP.as<float>(), dN.as<float>(), n_verts, rep.as<uint32_t>(), id.as<uint32_t>(), P2.as<double>(),
                                              N2.as<double>(), remap.as<uint32_t>());
  if (nt) weld_tri_keep<<<grid_of(nt), 256, 0, st>>>(dI.as<uint32_t>(), nt, remap.as<uint32_t>(), keep.as<uint32_t>());
  if (!scan_exclusive(keep.as<uint32_t>(), at.as<uint32_t>(), nt, tot.as<uint32_t>() + 1, st)) return VT_ERR_CUDA;
  if (nt)
    weld_tri_out<<<grid_of(nt), 256, 0, st>>>(dI.as<uint32_t>(), nt, remap.as<uint32_t>(), keep.as<uint32_t>(), at.as<uint32_t>(),
                                             I2.as<uint32_t>());
  if (cudaStreamSynchronize(st) != cudaSuccess) { cudaGetLastError(); return VT_ERR_CUDA; }
  const uint32_t nv2 = read_word(tot.as<uint32_t>()), nt2 = read_word(tot.as<uint32_t>() + 1);
  std::vector<double> hP, hN;
  std::vector<uint32_t> hI;
  if (!to_host(hP, P2.p, size_t(nv2) * 3) || !to_host(hN, N2.p, size_t(nv2) * 3) || !to_host(hI, I2.p, size_t(nt2) * 3)) return VT_ERR_CUDA;
  return vt::mesh_hand_out(std::move(hP), std::move(hN), std::move(hI), out);
}

vt_status vt_subdivide_device(int32_t device, const double* P, const double* N, uint32_t n_verts, const uint32_t* I, uint32_t n_idx, double h,
                              uint32_t max_passes, vt_mesh_out* out) {
  if (!out || (n_verts && (!P || !N)) || (n_idx && !I) || n_idx % 3 || !(h > 0)) return VT_ERR_ARG;
  *out = vt_mesh_out{};
  for (uint32_t k = 0; k < n_idx; k++) if (I[k] >= n_verts) return VT_ERR_ARG;
  if (!use_device(device)) return VT_ERR_NO_DEVICE;
  cudaStream_t st = 0;
  const double h2 = h * h;
  uint32_t nv = n_verts, nt = n_idx / 3;
  size_t vcap = std::max<size_t>(nv, 16);
  DevBuf dP, dN, tris, tris2;
  if (!dP.alloc(vcap * 24) || !dN.alloc(vcap * 24) || !tris.alloc(std::max<size_t>(nt, 16) * 12)) return VT_ERR_OOM;
  if (cudaMemcpy(dP.p, P, size_t(nv) * 24, cudaMemcpyHostToDevice) != cudaSuccess || cudaMemcpy(dN.p, N, size_t(nv) * 24, cudaMemcpyHostToDevice) != cudaSuccess ||
      (n_idx && cudaMemcpy(tris.p, I, size_t(n_idx) * 4, cudaMemcpyHostToDevice) != cudaSuccess))
    return VT_ERR_CUDA;
  for (uint32_t pass = 0; pass < max_passes && nt; pass++) {
    const uint32_t nc = 3 * nt, ns = pow2_at_least(nc);
    DevBuf items, ends, out_cnt, at, first, rank, call_id, tot;
    if (!items.alloc(size_t(ns) * sizeof(SortItem)) || !ends.alloc(size_t(nc) * 8) || !out_cnt.alloc(size_t(nt) * 4) || !at.alloc(size_t(nt) * 4) ||
        !first.alloc(size_t(nc) * 4) || !rank.alloc(size_t(nc) * 4) || !call_id.alloc(size_t(nc) * 4) || !tot.alloc(16))
      return VT_ERR_OOM;
    sub_calls<<<grid_of(nt), 256, 0, st>>>(dP.as<double>(), tris.as<uint32_t>(), nt, h2, items.as<SortItem>(), ends.as<uint2>(), out_cnt.as<uint32_t>());
    fill_items<<<grid_of(ns - nc), 256, 0, st>>>(items.as<SortItem>(), nc, ns);
    cudaMemsetAsync(first.p, 0, size_t(nc) * 4, st);
    bitonic_sort(items.as<SortItem>(), ns, st);
    sub_first<<<grid_of(nc), 256, 0, st>>>(items.as<SortItem>(), nc, first.as<uint32_t>());
    if (!scan_exclusive(first.as<uint32_t>(), rank.as<uint32_t>(), nc, tot.as<uint32_t>(), st) ||
        !scan_exclusive(out_cnt.as<uint32_t>(), at.as<uint32_t>(), nt, tot.as<uint32_t>() + 1, st))
      return VT_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) { cudaGetLastError(); return VT_ERR_CUDA; }
    const uint32_t n_new = read_word(tot.as<uint32_t>()), nt2 = read_word(tot.as<uint32_t>() + 1);
    if (n_new == 0) break;   // no edge longer than h: the triangles stay as they are
    if (size_t(nv) + n_new > vcap) {   // room for the new vertices, the old ones kept
      const size_t cap2 = std::max(size_t(nv) + n_new, vcap * 2);
      DevBuf nP, nN;
      if (!nP.alloc(cap2 * 24) || !nN.alloc(cap2 * 24)) return VT_ERR_OOM;
      if (cudaMemcpy(nP.p, dP.p, size_t(nv) * 24, cudaMemcpyDeviceToDevice) != cudaSuccess ||
          cudaMemcpy(nN.p, dN.p, size_t(nv) * 24, cudaMemcpyDeviceToDevice) != cudaSuccess)
        return VT_ERR_CUDA;
      std::swap(dP.p, nP.p);
      std::swap(dN.p, nN.p);
      vcap = cap2;
    }
    if (!tris2.alloc(std::max<size_t>(nt2, 16) * 12)) return VT_ERR_OOM;
    sub_assign<<<grid_of(nc), 256, 0, st>>>(items.as<SortItem>(), nc, rank.as<uint32_t>(), nv, ends.as<uint2>(), dP.as<double>(), dN.as<double>(),
                                            call_id.as<uint32_t>());
    sub_emit<<<grid_of(nt), 256, 0, st>>>(dP.as<double>(), tris.as<uint32_t>(), nt, h2, call_id.as<uint32_t>(), at.as<uint32_t>(),
                                          tris2.as<uint32_t>());
    if (cudaStreamSynchronize(st) != cudaSuccess) { cudaGetLastError(); return VT_ERR_CUDA; }
    std::swap(tris.p, tris2.p);
    nv += n_new;
    nt = nt2;
  }
  std::vector<double> hP, hN;
  std::vector<uint32_t> hI;
  if (!to_host(hP, dP.p, size_t(nv) * 3) || !to_host(hN, dN.p, size_t(nv) * 3) || !to_host(hI, tris.p, size_t(nt) * 3)) return VT_ERR_CUDA;
  return vt::mesh_hand_out(std::move(hP), std::move(hN), std::move(hI), out);
}

}  // extern "C"
