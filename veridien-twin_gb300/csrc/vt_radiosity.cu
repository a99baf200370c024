// Node radiosity on sm_103a: B = E + diag(rho) F B by Jacobi sweeps (the twin's jacobiGather + jacobiUpdate with
// Lambertian nodes, gpu/wgsl/kernels.wgsl.js:416-461), in plain FP32 on CUDA cores.
//
//   jacobi_matvec   one right-hand side: one warp per row, F streamed with 128-bit loads (HBM- or L2-bound: 4 B of F
//                   per 2 flops), B_in read from L1/L2; epilogue B_out = E + rho acc and the residual partials.
//   jacobi_matvec_tma  the same sweep with F's rows fed into shared memory by bulk copies (VT_PREC_FP32_TMA; ~20%
//                   slower than the plain kernel's 128-bit streaming loads on GB300, which stay the default).
//   jacobi_gemm     R right-hand sides (R <= 64): a 128 x 64 output tile per 256-thread block, 8 x 4 outputs per
//                   thread, F and B staged through double-buffered shared memory in 16-wide K slices, K split across
//                   blocks to fill the GPU. Compute-bound at 2 R flops per 4-byte element of F (R = 64: 32 flop/B)
//                   on the FP32 pipes.
// Every sweep also writes per-block sums of |B_out - B_in|^2 and |B_out|^2 in FP64; the relative update
// |B_out - B_in| / |B_out| is the relative residual |E + rho F B_in - B_in| / |B_out| of the Jacobi iterate.
#include <algorithm>

#include "vt_async.cuh"
#include "vt_kernels.cuh"

namespace vtk {
using namespace vtd;

constexpr int MV_THREADS = 256;

__device__ __forceinline__ void block_sum2(double a, double b, double* partials) {
  __shared__ double sa[32], sb[32];
  for (int o = 16; o > 0; o >>= 1) { a += __shfl_down_sync(0xffffffffu, a, o); b += __shfl_down_sync(0xffffffffu, b, o); }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (l == 0) { sa[w] = a; sb[w] = b; }
  __syncthreads();
  if (w == 0) {
    a = l < nw ? sa[l] : 0.0;
    b = l < nw ? sb[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) { a += __shfl_down_sync(0xffffffffu, a, o); b += __shfl_down_sync(0xffffffffu, b, o); }
    if (l == 0) { partials[2 * blockIdx.x] = a; partials[2 * blockIdx.x + 1] = b; }
  }
}

// KEEP: F fits in half the L2 and is read with the cache's default policy, so the next sweep finds it there; a larger F
// is streamed (evict-first), which keeps B and the vectors in L2 instead
template <bool KEEP>
__global__ void __launch_bounds__(MV_THREADS) jacobi_matvec_kernel(const float* __restrict__ F, const float* __restrict__ rho,
                                                                   const float* __restrict__ E, const float* __restrict__ Bin,
                                                                   float* __restrict__ Bout, uint32_t n, double* __restrict__ partials) {
  const uint32_t warps = MV_THREADS / 32;
  const uint32_t row = blockIdx.x * warps + (threadIdx.x >> 5);
  const uint32_t lane = threadIdx.x & 31u;
  double d2 = 0.0, b2 = 0.0;
  if (row < n) {
    const float* Fr = F + size_t(row) * n;
    float acc = 0.0f;
    // 128-bit loads only when every row starts 16-byte aligned (a caller's F may be an offset view)
    if ((n & 3u) == 0u && ((reinterpret_cast<uintptr_t>(F) | reinterpret_cast<uintptr_t>(Bin)) & 15u) == 0u) {
      const float4* F4 = reinterpret_cast<const float4*>(Fr);
      const float4* B4 = reinterpret_cast<const float4*>(Bin);
      const uint32_t n4 = n >> 2;
#pragma unroll 4
      for (uint32_t j = lane; j < n4; j += 32) {
        const float4 f = KEEP ? __ldg(F4 + j) : __ldcs(F4 + j);
        const float4 b = __ldg(B4 + j);
        acc = fmaf(f.x, b.x, acc); acc = fmaf(f.y, b.y, acc); acc = fmaf(f.z, b.z, acc); acc = fmaf(f.w, b.w, acc);
      }
    } else {
      for (uint32_t j = lane; j < n; j += 32) acc = fmaf(KEEP ? __ldg(Fr + j) : __ldcs(Fr + j), __ldg(Bin + j), acc);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const float b = fmaf(rho[row], acc, E[row]);
      Bout[row] = b;
      const double dd = double(b) - double(Bin[row]);
      d2 = dd * dd;
      b2 = double(b) * double(b);
    }
  }
  block_sum2(d2, b2, partials);
}

// ------------------------------------------------------------------------------------------ TMA-fed matvec
// One right-hand side, F rows streamed by the copy engine: thread 0 of each block keeps MVT_STAGES bulk copies
// (cp.async.bulk, 8 KB chunks of a row) in flight into a shared-memory ring, completing on mbarriers; all threads
// multiply a chunk from shared memory with B (L1/L2) while the next ones land. Each block takes rows blockIdx.x,
// blockIdx.x + gridDim.x, ...; a row's partial sums meet in a block reduction. Rows must start 16-byte aligned
// (n % 4 == 0). Every mbarrier wait is bounded (error flag, no hang).
constexpr int MVT_THREADS = 256, MVT_STAGES = 4;
constexpr uint32_t MVT_CHUNK = 2048;   // floats per bulk copy (8 KB)

__device__ uint32_t g_matvec_err;

__global__ void __launch_bounds__(MVT_THREADS) jacobi_matvec_tma_kernel(const float* __restrict__ F, const float* __restrict__ rho,
                                                                       const float* __restrict__ E, const float* __restrict__ Bin,
                                                                       float* __restrict__ Bout, uint32_t n, double* __restrict__ partials) {
  extern __shared__ __align__(128) float ring[];   // MVT_STAGES x MVT_CHUNK
  __shared__ __align__(8) uint64_t full[MVT_STAGES];
  __shared__ float red[MVT_THREADS / 32];
  using namespace async;
  const uint32_t tid = threadIdx.x;
  const uint32_t chunks = (n + MVT_CHUNK - 1) / MVT_CHUNK;
  const uint32_t rows = blockIdx.x < n ? (n - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
  const uint32_t items = rows * chunks;
  if (tid == 0) {
    for (int s = 0; s < MVT_STAGES; s++) mbar_init(smem_u32(full + s), 1);
    mbar_fence_init();
  }
  __syncthreads();
  auto issue = [&](uint32_t i) {
    const uint32_t s = i % MVT_STAGES, row = blockIdx.x + (i / chunks) * gridDim.x, c = i % chunks;
    const uint32_t bytes = min(MVT_CHUNK, n - c * MVT_CHUNK) * 4u;
    mbar_expect_tx(smem_u32(full + s), bytes);
    bulk_g2s(smem_u32(ring + s * MVT_CHUNK), F + size_t(row) * n + size_t(c) * MVT_CHUNK, bytes, smem_u32(full + s));
  };
  if (tid == 0)
    for (uint32_t i = 0; i < min(uint32_t(MVT_STAGES), items); i++) issue(i);
  float acc = 0.0f;
  double d2 = 0.0, b2 = 0.0;
  for (uint32_t i = 0; i < items; i++) {
    const uint32_t s = i % MVT_STAGES, c = i % chunks, row = blockIdx.x + (i / chunks) * gridDim.x;
    const bool ok = mbar_wait(smem_u32(full + s), (i / MVT_STAGES) & 1u, &g_matvec_err);
    if (__syncthreads_or(!ok)) break;   // a copy that never lands: every thread stops
    const uint32_t cnt4 = min(MVT_CHUNK, n - c * MVT_CHUNK) / 4u;
    const float4* f4 = reinterpret_cast<const float4*>(ring + s * MVT_CHUNK);
    const float4* b4 = reinterpret_cast<const float4*>(Bin + size_t(c) * MVT_CHUNK);
    for (uint32_t k = tid; k < cnt4; k += MVT_THREADS) {
      const float4 f = f4[k], b = __ldg(b4 + k);
      acc = fmaf(f.x, b.x, acc); acc = fmaf(f.y, b.y, acc); acc = fmaf(f.z, b.z, acc); acc = fmaf(f.w, b.w, acc);
    }
    __syncthreads();   // stage s read by every thread: it may be refilled
    if (tid == 0 && i + MVT_STAGES < items) issue(i + MVT_STAGES);
    if (c == chunks - 1) {
      float a = acc;
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if ((tid & 31u) == 0) red[tid >> 5] = a;
      __syncthreads();
      if (tid == 0) {
        float t = 0.0f;
        for (int w = 0; w < MVT_THREADS / 32; w++) t += red[w];
        const float b = fmaf(rho[row], t, E[row]);
        Bout[row] = b;
        const double dd = double(b) - double(Bin[row]);
        d2 += dd * dd;
        b2 += double(b) * double(b);
      }
      __syncthreads();
      acc = 0.0f;
    }
  }
  block_sum2(d2, b2, partials);
}

uint32_t jacobi_matvec_tma_blocks(uint32_t n) {
  static std::atomic<int> grid[MAX_DEVICES];
  const int g = per_device_value(grid, [](int dev) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, jacobi_matvec_tma_kernel, MVT_THREADS, MVT_STAGES * MVT_CHUNK * 4);
    return device_sms(dev) * std::max(per, 1);
  });
  return std::max(1u, std::min(n, uint32_t(g)));
}

void launch_jacobi_matvec_tma(const float* F, const float* rho, const float* E, const float* Bin, float* Bout, uint32_t n, double* partials,
                              uint32_t* n_partials, cudaStream_t st) {
  const uint32_t blocks = jacobi_matvec_tma_blocks(n);
  *n_partials = blocks;
  jacobi_matvec_tma_kernel<<<blocks, MVT_THREADS, MVT_STAGES * MVT_CHUNK * 4, st>>>(F, rho, E, Bin, Bout, n, partials);
}

uint32_t matvec_error(cudaStream_t st, bool reset) {
  uint32_t e = 0;
  cudaMemcpyFromSymbolAsync(&e, g_matvec_err, 4, 0, cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  if (reset && e) {
    const uint32_t z = 0;
    cudaMemcpyToSymbolAsync(g_matvec_err, &z, 4, 0, cudaMemcpyHostToDevice, st);
    cudaStreamSynchronize(st);
  }
  return e;
}

void launch_jacobi_matvec(const float* F, const float* rho, const float* E, const float* Bin, float* Bout, uint32_t n, double* partials,
                          uint32_t* n_partials, cudaStream_t st) {
  const uint32_t blocks = (n + MV_THREADS / 32 - 1) / (MV_THREADS / 32);
  *n_partials = blocks;
  static std::atomic<int> l2[MAX_DEVICES];
  const size_t l2_bytes = size_t(per_device_value(l2, [](int dev) {
    int b = 0;
    if (cudaDeviceGetAttribute(&b, cudaDevAttrL2CacheSize, dev) != cudaSuccess) { cudaGetLastError(); b = 0; }
    return b;
  }));
  if (size_t(n) * n * 4 <= l2_bytes / 2) jacobi_matvec_kernel<true><<<blocks, MV_THREADS, 0, st>>>(F, rho, E, Bin, Bout, n, partials);
  else jacobi_matvec_kernel<false><<<blocks, MV_THREADS, 0, st>>>(F, rho, E, Bin, Bout, n, partials);
}

// ---------------------------------------------------------------------------------------------- FP32 GEMM sweep
// 128 x 64 output tile per 256-thread block (8 x 4 outputs per thread), K in 16-wide slices double-buffered through
// shared memory: the next slice's F and B loads are in flight in registers while the current slice is multiplied.
// K is split over `splits` blocks per row tile so the grid fills the 152 SMs several times over; the split partial
// products are summed in split order by the combine kernel, which also applies the Jacobi update.
constexpr int GM = 128, GN = 64, GK = 16, G_THREADS = 256;

template <bool SPLIT>
__global__ void __launch_bounds__(G_THREADS) jacobi_gemm_fp32_kernel(const float* __restrict__ F, const float* __restrict__ rho,
                                                                     const float* __restrict__ E, const float* __restrict__ Bin,
                                                                     float* __restrict__ Bout, uint32_t n, uint32_t R, uint32_t kchunk,
                                                                     float* __restrict__ part, double* __restrict__ partials) {
  __shared__ __align__(16) float As[2][GK][GM + 4];   // F slices, transposed: As[b][k][m]
  __shared__ __align__(16) float Bs[2][GK][GN];       // B slices: Bs[b][k][c]
  const uint32_t tid = threadIdx.x;
  const uint32_t row0 = blockIdx.x * GM;
  const uint32_t kbeg = blockIdx.y * kchunk, kend = min(n, kbeg + kchunk);
  const uint32_t tm = tid / 16, tn = tid % 16;      // 16 x 16 threads, each 8 rows x 4 cols
  const bool vec = (n & 3u) == 0u && (reinterpret_cast<uintptr_t>(F) & 15u) == 0u;   // 16-byte aligned rows
  float acc[8][4];
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0f;
  float4 fa[2], fb;
  // F slice 128 x 16: 512 float4, 2 per thread; B slice 16 x 64: 256 float4, 1 per thread (columns >= R are zero)
  auto load = [&](uint32_t k0) {
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const uint32_t idx = tid + q * G_THREADS;
      const uint32_t r = idx / (GK / 4), c4 = idx % (GK / 4);
      const uint32_t gr = row0 + r, gk = k0 + c4 * 4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gr < n) {
        const float* p = F + size_t(gr) * n;
        if (vec && gk + 3 < kend) v = __ldcs(reinterpret_cast<const float4*>(p + gk));   // 16-byte aligned rows
        else {
          v.x = gk < kend ? p[gk] : 0.f; v.y = gk + 1 < kend ? p[gk + 1] : 0.f; v.z = gk + 2 < kend ? p[gk + 2] : 0.f;
          v.w = gk + 3 < kend ? p[gk + 3] : 0.f;
        }
      }
      fa[q] = v;
    }
    const uint32_t r = tid / (GN / 4), c4 = tid % (GN / 4);
    const uint32_t gk = k0 + r, gc = c4 * 4;
    fb = (gk < kend && gc < R) ? __ldg(reinterpret_cast<const float4*>(Bin + size_t(gk) * R + gc)) : make_float4(0.f, 0.f, 0.f, 0.f);
  };
  auto store = [&](int b) {
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const uint32_t idx = tid + q * G_THREADS;
      const uint32_t r = idx / (GK / 4), c4 = idx % (GK / 4);
      As[b][c4 * 4 + 0][r] = fa[q].x; As[b][c4 * 4 + 1][r] = fa[q].y; As[b][c4 * 4 + 2][r] = fa[q].z; As[b][c4 * 4 + 3][r] = fa[q].w;
    }
    *reinterpret_cast<float4*>(&Bs[b][tid / (GN / 4)][(tid % (GN / 4)) * 4]) = fb;
  };
  load(kbeg);
  store(0);
  __syncthreads();
  int buf = 0;
  for (uint32_t k0 = kbeg; k0 < kend; k0 += GK) {
    const bool more = k0 + GK < kend;
    if (more) load(k0 + GK);
#pragma unroll
    for (int k = 0; k < GK; k++) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][k][tm * 8]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][k][tm * 8 + 4]);
      const float4 b = *reinterpret_cast<const float4*>(&Bs[buf][k][tn * 4]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], bb[j], acc[i][j]);
    }
    if (more) store(buf ^ 1);
    __syncthreads();
    buf ^= 1;
  }
  if (SPLIT) {
    // partial product of this K range: part[split][row][col]
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const uint32_t gr = row0 + tm * 8 + i, gc = tn * 4;
      if (gr >= n || gc >= R) continue;
      *reinterpret_cast<float4*>(part + (size_t(blockIdx.y) * n + gr) * R + gc) = make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
    }
    return;
  }
  double d2 = 0.0, b2 = 0.0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint32_t gr = row0 + tm * 8 + i;
    if (gr >= n) continue;
    const float rr = rho[gr];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const uint32_t gc = tn * 4 + j;
      if (gc >= R) continue;
      const size_t o = size_t(gr) * R + gc;
      const float b = fmaf(rr, acc[i][j], E[o]);
      Bout[o] = b;
      const double dd = double(b) - double(Bin[o]);
      d2 += dd * dd;
      b2 += double(b) * double(b);
    }
  }
  block_sum2(d2, b2, partials);
}

// B_out = E + rho (sum over splits of the partial products, in split order), and the residual partials
__global__ void __launch_bounds__(256) jacobi_gemm_combine_kernel(const float* __restrict__ part, uint32_t splits, const float* __restrict__ rho,
                                                                  const float* __restrict__ E, const float* __restrict__ Bin,
                                                                  float* __restrict__ Bout, uint32_t n, uint32_t R, double* __restrict__ partials) {
  const size_t total = size_t(n) * R / 4, stride = size_t(n) * R / 4;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double d2 = 0.0, b2 = 0.0;
  if (i < total) {
    const float4* P = reinterpret_cast<const float4*>(part);
    float4 a = P[i];
    for (uint32_t s = 1; s < splits; s++) {
      const float4 v = P[s * stride + i];
      a.x += v.x; a.y += v.y; a.z += v.z; a.w += v.w;
    }
    const float rr = rho[(i * 4) / R];
    const float4 e = reinterpret_cast<const float4*>(E)[i], bi = reinterpret_cast<const float4*>(Bin)[i];
    const float4 b = make_float4(fmaf(rr, a.x, e.x), fmaf(rr, a.y, e.y), fmaf(rr, a.z, e.z), fmaf(rr, a.w, e.w));
    reinterpret_cast<float4*>(Bout)[i] = b;
    const double dx = double(b.x) - bi.x, dy = double(b.y) - bi.y, dz = double(b.z) - bi.z, dw = double(b.w) - bi.w;
    d2 = dx * dx + dy * dy + dz * dz + dw * dw;
    b2 = double(b.x) * b.x + double(b.y) * b.y + double(b.z) * b.z + double(b.w) * b.w;
  }
  block_sum2(d2, b2, partials);
}

namespace {
uint32_t gemm_splits(uint32_t n, int sms) {
  const uint32_t tiles = (n + GM - 1) / GM;
  const uint32_t want = uint32_t(8 * std::max(sms, 1));   // about 8 blocks per SM in flight over the sweep
  uint32_t s = std::max(1u, std::min(16u, (want + tiles - 1) / tiles));
  while (s > 1 && (n + s - 1) / s < 4 * GK) s--;          // at least 64 columns of F per split
  return s;
}
int sm_count() {
  static std::atomic<int> sms[MAX_DEVICES];
  return per_device_value(sms, device_sms);
}
}  // namespace

size_t jacobi_gemm_fp32_work(uint32_t n, uint32_t R) {
  const uint32_t s = gemm_splits(n, sm_count());
  return s > 1 ? size_t(s) * n * R * 4 : 0;
}

void launch_jacobi_gemm_fp32(const float* F, const float* rho, const float* E, const float* Bin, float* Bout, uint32_t n, uint32_t R,
                             float* work, double* partials, uint32_t* n_partials, cudaStream_t st) {
  const uint32_t tiles = (n + GM - 1) / GM;
  const uint32_t s = work ? gemm_splits(n, sm_count()) : 1u;
  const uint32_t kchunk = s > 1 ? ((n + s - 1) / s + GK - 1) / GK * GK : n;
  const uint32_t splits = (n + kchunk - 1) / kchunk;
  if (splits <= 1) {
    *n_partials = tiles;
    jacobi_gemm_fp32_kernel<false><<<dim3(tiles, 1), G_THREADS, 0, st>>>(F, rho, E, Bin, Bout, n, R, n, nullptr, partials);
    return;
  }
  jacobi_gemm_fp32_kernel<true><<<dim3(tiles, splits), G_THREADS, 0, st>>>(F, rho, E, Bin, Bout, n, R, kchunk, work, partials);
  const uint32_t blocks = uint32_t((size_t(n) * R / 4 + 255) / 256);
  *n_partials = blocks;
  jacobi_gemm_combine_kernel<<<blocks, 256, 0, st>>>(work, splits, rho, E, Bin, Bout, n, R, partials);
}

__global__ void reduce_partials_kernel(const double* __restrict__ p, uint32_t n, double* __restrict__ out) {
  double a = 0.0, b = 0.0;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) { a += p[2 * i]; b += p[2 * i + 1]; }
  __shared__ double sa[1024], sb[1024];
  sa[threadIdx.x] = a; sb[threadIdx.x] = b;
  __syncthreads();
  for (uint32_t s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) { sa[threadIdx.x] += sa[threadIdx.x + s]; sb[threadIdx.x] += sb[threadIdx.x + s]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { out[0] = sa[0]; out[1] = sb[0]; }
}

void launch_reduce_partials(const double* partials, uint32_t n, double* out, cudaStream_t st) {
  reduce_partials_kernel<<<1, 1024, 0, st>>>(partials, n, out);
}

// ---------------------------------------------------------------------------------------------- form factors
// F_ij = A_j max(0, n_i.w) max(0, -n_j.w) / (pi r^2 + A_j) (disk approximation), F_ii = 0, each row scaled to a
// sum <= 1. One block per row: the row sum in FP64 first, then the scaled row written.
__global__ void form_factor_kernel(uint32_t n, const float* __restrict__ C, const float* __restrict__ N, const float* __restrict__ A,
                                   float* __restrict__ F) {
  const uint32_t i = blockIdx.x;
  const float cx = C[3 * i], cy = C[3 * i + 1], cz = C[3 * i + 2];
  const float nx = N[3 * i], ny = N[3 * i + 1], nz = N[3 * i + 2];
  auto ff = [&](uint32_t j) -> double {
    if (j == i) return 0.0;
    const double wx = double(C[3 * j]) - cx, wy = double(C[3 * j + 1]) - cy, wz = double(C[3 * j + 2]) - cz;
    const double r2 = wx * wx + wy * wy + wz * wz;
    const double r = sqrt(r2);
    if (!(r > 0.0)) return 0.0;
    const double ci = (nx * wx + ny * wy + nz * wz) / r;
    const double cj = -(N[3 * j] * wx + N[3 * j + 1] * wy + N[3 * j + 2] * wz) / r;
    if (ci <= 0.0 || cj <= 0.0) return 0.0;
    return double(A[j]) * ci * cj / (3.14159265358979323846 * r2 + double(A[j]));
  };
  double s = 0.0;
  for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) s += ff(j);
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  const double sc = red[0] > 1.0 ? 1.0 / red[0] : 1.0;
  for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) F[size_t(i) * n + j] = float(ff(j) * sc);
}

void launch_form_factors(uint32_t n, const float* C, const float* N, const float* A, float* F, cudaStream_t st) {
  if (!n) return;
  form_factor_kernel<<<n, 256, 0, st>>>(n, C, N, A, F);
}

// ------------------------------------------------------------------------------------- form factors with visibility
// F_ij = (disk form factor of the centres) x V_ij, V_ij the fraction of K stratified rays between points of the two
// patch discs that no surface of the scene blocks (the gather of gpu/wgsl/kernels.wgsl.js:271 gatherDir, dense),
// then each row scaled to a sum <= 1. A patch is a disc of its area around its centre, tangent to its normal; ray
// k joins the points of the discs' half radius at Kronecker sample k (each disc its own shift), each lifted along
// its normal by 5 mm + a tenth of that radius (so that a tangent disc on a curved, faceted surface starts in front
// of it). V is symmetric: each unordered pair is traced once, on persistent traversal lanes.
constexpr int FV_THREADS = 256;

__device__ __forceinline__ float3 disc_point(const float* C, const float* N, const float* A, uint32_t i, float u, float v) {
  const float3 c = f3(C[3 * i], C[3 * i + 1], C[3 * i + 2]), nn = f3(N[3 * i], N[3 * i + 1], N[3 * i + 2]);
  const float rh = 0.5f * sqrtf(A[i] * INV_PI_F), r = rh * sqrtf(u);
  float sp, cp;
  sincosf(2.0f * PI_F * v, &sp, &cp);
  return c + basis_t(nn) * (r * cp) + basis_b(nn) * (r * sp) + nn * (5e-3f + 0.1f * rh);
}
__device__ __forceinline__ bool facing(const float* C, const float* N, uint32_t i, uint32_t j) {
  const float wx = C[3 * j] - C[3 * i], wy = C[3 * j + 1] - C[3 * i + 1], wz = C[3 * j + 2] - C[3 * i + 2];
  return N[3 * i] * wx + N[3 * i + 1] * wy + N[3 * i + 2] * wz > 0.0f && N[3 * j] * wx + N[3 * j + 1] * wy + N[3 * j + 2] * wz < 0.0f;
}

__global__ void __launch_bounds__(FV_THREADS, 4) ff_visibility_kernel(const Scene S, const float* __restrict__ C, const float* __restrict__ N,
                                                                     const float* __restrict__ A, uint32_t n, uint32_t K, uint32_t* head,
                                                                     uint8_t* __restrict__ counts) {
  __shared__ uint2 stack_sh[SH_DEPTH * FV_THREADS];
  LaneStack stk;
  stk.sh = stack_sh; stk.lane = threadIdx.x; stk.stride = FV_THREADS;
  TraceState st;
  const uint32_t skip = ldu(S.su + 7);
  const uint32_t total = n * n;
  float3 o = f3(0, 0, 0), d = f3(0, 0, 1);
  uint32_t i = 0, j = 0, k = 0, vis = 0;
  bool active = false, exhausted = false;
  auto next_ray = [&]() -> bool {
    for (; k < K; k++) {
      const float3 a = disc_point(C, N, A, i, kr(k, R2A, 0.5f), kr(k, R2B, 0.5f));
      const float3 b = disc_point(C, N, A, j, kr(k, R2A, 0.25f), kr(k, R2B, 0.75f));
      const float3 w = b - a;
      const float dist = length(w);
      if (!(dist > 2e-4f)) { vis++; continue; }
      o = a;
      d = w / dist;
      st.best = Hit{dist - 1e-4f, 0.0f, 0.0f, MISS, MISS};
      if (trace_phase(S, 0u, o, d, 0.0f, 0.5f, 3u, skip, st, -1)) return true;
      vis++;
    }
    return false;
  };
  auto finish = [&]() {
    counts[size_t(i) * n + j] = uint8_t(vis);
    counts[size_t(j) * n + i] = uint8_t(vis);
    active = false;
  };
  auto start = [&](uint32_t idx) {
    i = idx / n;
    j = idx % n;
    if (j <= i) return;
    if (!facing(C, N, i, j)) { vis = 0; finish(); return; }
    k = 0;
    vis = 0;
    active = true;
    if (!next_ray()) finish();
  };
  while (take_rays(active, exhausted, head, total, REFILL, start)) {
    if (!active) continue;
    const int r = trace_step<true>(S, 0.0f, st, stk);
    bool done = r == 2;
    if (r == 1) done = !trace_phase(S, 0u, o, d, 0.0f, 0.5f, 3u, skip, st, st.k + 1);
    if (!done) continue;
    if (st.best.tri == MISS) vis++;
    k++;
    if (!next_ray()) finish();
  }
}

__global__ void ff_rows_kernel(uint32_t n, const float* __restrict__ C, const float* __restrict__ N, const float* __restrict__ A,
                               const uint8_t* __restrict__ counts, uint32_t K, float* __restrict__ F) {
  const uint32_t i = blockIdx.x;
  const float cx = C[3 * i], cy = C[3 * i + 1], cz = C[3 * i + 2];
  const float nx = N[3 * i], ny = N[3 * i + 1], nz = N[3 * i + 2];
  const double inv_k = 1.0 / double(K);
  auto ff = [&](uint32_t j) -> double {
    if (j == i) return 0.0;
    const uint8_t c = counts[size_t(i) * n + j];
    if (!c) return 0.0;
    const double wx = double(C[3 * j]) - cx, wy = double(C[3 * j + 1]) - cy, wz = double(C[3 * j + 2]) - cz;
    const double r2 = wx * wx + wy * wy + wz * wz;
    const double r = sqrt(r2);
    if (!(r > 0.0)) return 0.0;
    const double ci = (nx * wx + ny * wy + nz * wz) / r;
    const double cj = -(N[3 * j] * wx + N[3 * j + 1] * wy + N[3 * j + 2] * wz) / r;
    if (ci <= 0.0 || cj <= 0.0) return 0.0;
    return double(A[j]) * ci * cj / (3.14159265358979323846 * r2 + double(A[j])) * (double(c) * inv_k);
  };
  double s = 0.0;
  for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) s += ff(j);
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  const double sc = red[0] > 1.0 ? 1.0 / red[0] : 1.0;
  for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) F[size_t(i) * n + j] = float(ff(j) * sc);
}

void launch_form_factors_visible(const Scene& S, uint32_t n, const float* C, const float* N, const float* A, uint32_t K, uint32_t* head,
                                 uint8_t* counts, float* F, int blocks, cudaStream_t st) {
  if (!n) return;
  cudaMemsetAsync(counts, 0, size_t(n) * n, st);
  cudaMemsetAsync(head, 0, 4, st);
  ff_visibility_kernel<<<blocks, FV_THREADS, 0, st>>>(S, C, N, A, n, K, head, counts);
  ff_rows_kernel<<<n, 256, 0, st>>>(n, C, N, A, counts, K, F);
}

}  // namespace vtk
