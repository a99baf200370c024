// Node radiosity on sm_103a: B = E + diag(rho) F B by Jacobi sweeps (the twin's jacobiGather + jacobiUpdate with
// Lambertian nodes, gpu/wgsl/kernels.wgsl.js:416-461), in plain FP32 on CUDA cores.
//
//   jacobi_matvec   one right-hand side: one warp per row, F streamed with 128-bit loads (HBM- or L2-bound: 4 B of F
//                   per 2 flops), B_in read from L1/L2; epilogue B_out = E + rho acc and the residual partials.
//   jacobi_gemm     R right-hand sides (R <= 64): a 128 x 64 output tile per 256-thread block, 8 x 4 outputs per
//                   thread, F and B staged through shared memory in 32-wide K slices. Compute-bound at 2 R flops per
//                   4-byte element of F (R = 64: 32 flop/B) on the FP32 pipes.
// Every sweep also writes per-block sums of |B_out - B_in|^2 and |B_out|^2 in FP64; the relative update
// |B_out - B_in| / |B_out| is the relative residual |E + rho F B_in - B_in| / |B_out| of the Jacobi iterate.
#include "vt_kernels.cuh"

namespace vtk {

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
    if ((n & 3u) == 0u) {
      const float4* F4 = reinterpret_cast<const float4*>(Fr);
      const float4* B4 = reinterpret_cast<const float4*>(Bin);
      const uint32_t n4 = n >> 2;
#pragma unroll 4
      for (uint32_t j = lane; j < n4; j += 32) {
        const float4 f = __ldcs(F4 + j);
        const float4 b = __ldg(B4 + j);
        acc = fmaf(f.x, b.x, acc); acc = fmaf(f.y, b.y, acc); acc = fmaf(f.z, b.z, acc); acc = fmaf(f.w, b.w, acc);
      }
    } else {
      for (uint32_t j = lane; j < n; j += 32) acc = fmaf(__ldcs(Fr + j), __ldg(Bin + j), acc);
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

void launch_jacobi_matvec(const float* F, const float* rho, const float* E, const float* Bin, float* Bout, uint32_t n, double* partials,
                          uint32_t* n_partials, cudaStream_t st) {
  const uint32_t blocks = (n + MV_THREADS / 32 - 1) / (MV_THREADS / 32);
  *n_partials = blocks;
  jacobi_matvec_kernel<<<blocks, MV_THREADS, 0, st>>>(F, rho, E, Bin, Bout, n, partials);
}

// ---------------------------------------------------------------------------------------------- FP32 GEMM sweep
constexpr int GM = 128, GN = 64, GK = 32, G_THREADS = 256;

__global__ void __launch_bounds__(G_THREADS) jacobi_gemm_fp32_kernel(const float* __restrict__ F, const float* __restrict__ rho,
                                                                     const float* __restrict__ E, const float* __restrict__ Bin,
                                                                     float* __restrict__ Bout, uint32_t n, uint32_t R,
                                                                     double* __restrict__ partials) {
  __shared__ __align__(16) float As[GK][GM + 4];   // F tile, transposed: As[k][m]
  __shared__ __align__(16) float Bs[GK][GN];       // B tile: Bs[k][c]
  const uint32_t tid = threadIdx.x;
  const uint32_t row0 = blockIdx.x * GM;
  const uint32_t tm = tid / 16, tn = tid % 16;      // 16 x 16 threads, each 8 rows x 4 cols
  float acc[8][4];
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0f;
  for (uint32_t k0 = 0; k0 < n; k0 += GK) {
    // F tile 128 x 32: 1024 float4, 4 per thread
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint32_t idx = tid + q * G_THREADS;         // 0..1023
      const uint32_t r = idx / (GK / 4), c4 = idx % (GK / 4);
      const uint32_t gr = row0 + r, gk = k0 + c4 * 4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gr < n) {
        const float* p = F + size_t(gr) * n;
        if ((n & 3u) == 0u && gk + 3 < n) v = __ldcs(reinterpret_cast<const float4*>(p + gk));   // 16-byte aligned rows
        else {
          v.x = gk < n ? p[gk] : 0.f; v.y = gk + 1 < n ? p[gk + 1] : 0.f; v.z = gk + 2 < n ? p[gk + 2] : 0.f;
          v.w = gk + 3 < n ? p[gk + 3] : 0.f;
        }
      }
      As[c4 * 4 + 0][r] = v.x; As[c4 * 4 + 1][r] = v.y; As[c4 * 4 + 2][r] = v.z; As[c4 * 4 + 3][r] = v.w;
    }
    // B tile 32 x 64: 512 float4, 2 per thread (columns >= R are zero)
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const uint32_t idx = tid + q * G_THREADS;
      const uint32_t r = idx / (GN / 4), c4 = idx % (GN / 4);
      const uint32_t gk = k0 + r, gc = c4 * 4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gk < n && gc < R) v = __ldg(reinterpret_cast<const float4*>(Bin + size_t(gk) * R + gc));
      *reinterpret_cast<float4*>(&Bs[r][gc]) = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < GK; k++) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[k][tm * 8]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[k][tm * 8 + 4]);
      const float4 b = *reinterpret_cast<const float4*>(&Bs[k][tn * 4]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], bb[j], acc[i][j]);
    }
    __syncthreads();
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

void launch_jacobi_gemm_fp32(const float* F, const float* rho, const float* E, const float* Bin, float* Bout, uint32_t n, uint32_t R,
                             double* partials, uint32_t* n_partials, cudaStream_t st) {
  const uint32_t blocks = (n + GM - 1) / GM;
  *n_partials = blocks;
  jacobi_gemm_fp32_kernel<<<blocks, G_THREADS, 0, st>>>(F, rho, E, Bin, Bout, n, R, partials);
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

}  // namespace vtk
