// Multi-right-hand-side node radiosity sweeps on the 5th-generation tensor cores (tcgen05) of sm_103a.
//
// tc_gemm_kernel: one CTA computes a 128-row x 64-column FP32 accumulator in tensor memory (TMEM) over one split of
// the K range. Warp 0 lane 0 feeds a ring of shared-memory stages with TMA (cp.async.bulk.tensor, 128-byte
// swizzle; a stage is 128 rows x 128 B of F and 64 rows x 128 B of the transposed right-hand sides Bt), warp 1
// lane 0 issues tcgen05.mma (M = 128, N = 64, K = 16 bf16 / 32 e4m3 per instruction) and releases each stage with
// tcgen05.commit, and all four warps read the accumulator back with tcgen05.ld into per-split partial sums. The
// combine kernels (CUDA cores, HBM-bound and small) apply the Jacobi epilogue or the accurate residual in FP64.
//
// The sweep streams F once: 2 B per element in BF16, 1 B in FP8, so it is HBM-bound (64 flop/B at 64 right-hand
// sides in BF16, 128 in FP8, both under the tensor ridge). Every wait on an mbarrier is bounded by a clock limit:
// a wait that runs out sets *err and the kernel drains its TMA copies, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "vt_async.cuh"
#include "vt_tc.cuh"

namespace vtk {

namespace {

constexpr int TC_THREADS = 128;
constexpr uint32_t A_BYTES = 128 * 128;   // 128 rows x 128 B
constexpr uint32_t B_BYTES = 64 * 128;    // 64 rows x 128 B
using namespace async;

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const TcMap* map, int32_t c0, int32_t c1, uint32_t bar) {
  asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms 1024 B apart
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = uint64_t((saddr & 0x3FFFFu) >> 4);
  d |= uint64_t(1) << 16;                 // leading byte offset (unused for swizzled K-major)
  d |= uint64_t(1024 >> 4) << 32;         // stride byte offset: one 8-row atom
  d |= uint64_t(1) << 46;                 // descriptor version
  d |= uint64_t(2) << 61;                 // 128-byte swizzle
  return d;
}
// instruction descriptor: D f32, A/B type, K-major A and B, N = 64, M = 128
__host__ __device__ constexpr uint32_t idesc_of(uint32_t ab_type) {
  return (1u << 4) | (ab_type << 7) | (ab_type << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
}
constexpr uint32_t IDESC_BF16 = idesc_of(1);   // kind::f16, bf16 x bf16
constexpr uint32_t IDESC_E4M3 = idesc_of(0);   // kind::f8f6f4, e4m3 x e4m3

template <int MODE>
__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  if (MODE == TC_FP8) {
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                 "l"(a), "l"(b), "r"(IDESC_E4M3), "r"(accumulate)
                 : "memory");
  } else {
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                 "l"(a), "l"(b), "r"(IDESC_BF16), "r"(accumulate)
                 : "memory");
  }
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

template <int MODE, int STAGES>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ TcMap mA, const __grid_constant__ TcMap mA2, const __grid_constant__ TcMap mB,
                   const __grid_constant__ TcMap mB2, uint32_t n, uint32_t k_tiles, float* __restrict__ partials, uint32_t* err) {
  constexpr bool X3 = MODE == TC_BF16X3;
  constexpr uint32_t STAGE_BYTES = (X3 ? 2 : 1) * (A_BYTES + B_BYTES);
  constexpr uint32_t K_ELEMS = MODE == TC_FP8 ? 128 : 64;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);   // full[STAGES], empty[STAGES], done
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const uint32_t m0 = blockIdx.x * 128u;
  const uint32_t split = blockIdx.y;
  const uint32_t total_kt = (n + K_ELEMS - 1) / K_ELEMS;
  const uint32_t kt0 = split * k_tiles;
  const uint32_t kt1 = min(total_kt, kt0 + k_tiles);
  const uint32_t nkt = kt1 > kt0 ? kt1 - kt0 : 0u;
  auto full = [&](uint32_t s) { return smem_u32(bars + s); };
  auto empty = [&](uint32_t s) { return smem_u32(bars + STAGES + s); };
  const uint32_t done = smem_u32(bars + 2 * STAGES);
  auto sA = [&](uint32_t s) { return smem_u32(smem + s * STAGE_BYTES); };
  auto sA2 = [&](uint32_t s) { return smem_u32(smem + s * STAGE_BYTES + A_BYTES); };
  auto sB = [&](uint32_t s) { return smem_u32(smem + s * STAGE_BYTES + (X3 ? 2 : 1) * A_BYTES); };
  auto sB2 = [&](uint32_t s) { return smem_u32(smem + s * STAGE_BYTES + 2 * A_BYTES + B_BYTES); };

  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < STAGES; s++) { mbar_init(full(s), 1); mbar_init(empty(s), 1); }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(tmem_slot)) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // TMA producer
    uint32_t issued = 0;
    for (uint32_t kt = 0; kt < nkt; kt++) {
      const uint32_t s = kt % STAGES;
      if (kt >= STAGES && !mbar_wait(empty(s), ((kt / STAGES) & 1u) ^ 1u, err)) break;
      mbar_expect_tx(full(s), STAGE_BYTES);
      const int32_t kx = int32_t((kt0 + kt) * K_ELEMS);
      tma_load_2d(sA(s), &mA, kx, int32_t(m0), full(s));
      if (X3) tma_load_2d(sA2(s), &mA2, kx, int32_t(m0), full(s));
      tma_load_2d(sB(s), &mB, kx, 0, full(s));
      if (X3) tma_load_2d(sB2(s), &mB2, kx, 0, full(s));
      issued++;
    }
    // drain: every stage this thread filled must have landed before the CTA may exit
    for (uint32_t kt = issued > STAGES ? issued - STAGES : 0; kt < issued; kt++) mbar_wait(full(kt % STAGES), (kt / STAGES) & 1u, err);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    bool ok = true;
    for (uint32_t kt = 0; kt < nkt && ok; kt++) {
      const uint32_t s = kt % STAGES;
      ok = mbar_wait(full(s), (kt / STAGES) & 1u, err);
      if (!ok) break;
      tc_fence_after();
#pragma unroll
      for (uint32_t k = 0; k < 4; k++) {   // 4 MMAs of 32 bytes of K each
        const uint64_t a = sw128_desc(sA(s) + 32 * k), b = sw128_desc(sB(s) + 32 * k);
        mma<MODE>(tmem, a, b, (kt | k) != 0u);
        if (X3) {
          mma<MODE>(tmem, a, sw128_desc(sB2(s) + 32 * k), 1u);
          mma<MODE>(tmem, sw128_desc(sA2(s) + 32 * k), b, 1u);
        }
      }
      mma_commit(empty(s));
    }
    if (nkt > 0 && ok) mma_commit(done);
    else mbar_arrive(done);
  }
  __syncwarp();
  // epilogue: warp w reads accumulator rows 32 w .. 32 w + 31 (TMEM lanes), 64 columns
  const bool have = mbar_wait(done, 0, err) && nkt > 0;
  __syncwarp();   // tcgen05.ld is warp-collective
  tc_fence_after();
  float v[64];
#pragma unroll
  for (int c = 0; c < 4; c++) tmem_ld16(tmem + ((warp * 32u) << 16) + 16u * c, v + 16 * c);
  const uint32_t row = m0 + warp * 32u + lane;
  if (row < n) {
    float4* dst = reinterpret_cast<float4*>(partials + (size_t(split) * n + row) * 64);
#pragma unroll
    for (int c = 0; c < 16; c++)
      dst[c] = have ? make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
}

template <int MODE, int STAGES>
constexpr size_t smem_bytes() {
  return size_t(STAGES) * (MODE == TC_BF16X3 ? 2 : 1) * (A_BYTES + B_BYTES) + 1024 + 8 * (2 * STAGES + 1) + 16;
}

template <int MODE, int STAGES>
void launch_gemm(const TcMap* A, const TcMap* A2, const TcMap* B, const TcMap* B2, uint32_t n, uint32_t splits, uint32_t k_tiles,
                 float* partials, uint32_t* err, cudaStream_t st) {
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(tc_gemm_kernel<MODE, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_bytes<MODE, STAGES>()));
  });
  const dim3 grid((n + 127) / 128, splits);
  tc_gemm_kernel<MODE, STAGES><<<grid, TC_THREADS, smem_bytes<MODE, STAGES>(), st>>>(*A, A2 ? *A2 : *A, *B, B2 ? *B2 : *B, n, k_tiles,
                                                                                    partials, err);
}

// ------------------------------------------------------------------------------------------------ CUDA-core helpers
__global__ void split_bf16_kernel(const float* __restrict__ F, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, size_t count) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += size_t(gridDim.x) * blockDim.x) {
    const float f = F[i];
    const __nv_bfloat16 h = __float2bfloat16_rn(f);
    hi[i] = h;
    lo[i] = __float2bfloat16_rn(f - __bfloat162float(h));
  }
}

__device__ __forceinline__ float block_max(float v) {
  __shared__ float red[32];
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < int(blockDim.x >> 5) ? red[l] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (l == 0) red[0] = v;
  }
  __syncthreads();
  const float r = red[0];
  __syncthreads();
  return r;
}

// one block per row: s_i = max_j |F_ij| / 448 (the largest finite e4m3), q_ij = e4m3(F_ij / s_i)
__global__ void quant_rows_fp8_kernel(const float* __restrict__ F, uint8_t* __restrict__ q, float* __restrict__ row_scale, uint32_t n) {
  const size_t base = size_t(blockIdx.x) * n;
  float m = 0.0f;
  for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) m = fmaxf(m, fabsf(F[base + j]));
  m = block_max(m);
  const float s = m > 0.0f ? m / 448.0f : 1.0f;
  if (threadIdx.x == 0) row_scale[blockIdx.x] = s;
  const float inv = 1.0f / s;
  for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
    const __nv_fp8_e4m3 e(F[base + j] * inv);
    q[base + j] = *reinterpret_cast<const uint8_t*>(&e);
  }
}

// column maxima of X (n x R) for the FP8 column scales (positive floats compare as their bit patterns)
__global__ void col_max_kernel(const float* __restrict__ X, uint32_t n, uint32_t R, uint32_t* __restrict__ col_max) {
  const uint32_t c = threadIdx.x % 64u;
  float m = 0.0f;
  if (c < R)
    for (uint32_t i = blockIdx.x * (blockDim.x / 64u) + threadIdx.x / 64u; i < n; i += gridDim.x * (blockDim.x / 64u))
      m = fmaxf(m, fabsf(X[size_t(i) * R + c]));
  if (c < R && m > 0.0f) atomicMax(col_max + c, __float_as_uint(m));
}

// X (n x R) -> Bt (64 x n): transposed through a 32 x 32 shared tile; rows c >= R of Bt are zero
template <int MODE>
__global__ void pack_b_kernel(const float* __restrict__ X, uint32_t n, uint32_t R, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                              uint8_t* __restrict__ q8, const uint32_t* __restrict__ col_max, float* __restrict__ col_scale) {
  __shared__ float tile[32][33];
  const uint32_t i0 = blockIdx.x * 32u, c0 = blockIdx.y * 32u;
  for (uint32_t k = threadIdx.y; k < 32u; k += blockDim.y) {
    const uint32_t i = i0 + k, c = c0 + threadIdx.x;
    tile[k][threadIdx.x] = (i < n && c < R) ? X[size_t(i) * R + c] : 0.0f;
  }
  __syncthreads();
  for (uint32_t k = threadIdx.y; k < 32u; k += blockDim.y) {
    const uint32_t c = c0 + k, i = i0 + threadIdx.x;
    if (i >= n) continue;
    const float x = tile[threadIdx.x][k];
    const size_t o = size_t(c) * n + i;
    if (MODE == TC_FP8) {
      const float m = c < R ? __uint_as_float(col_max[c]) : 0.0f;
      const float s = m > 0.0f ? m / 448.0f : 1.0f;
      if (blockIdx.x == 0 && threadIdx.x == 0) col_scale[c] = s;
      const __nv_fp8_e4m3 e(x / s);
      q8[o] = *reinterpret_cast<const uint8_t*>(&e);
    } else {
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      hi[o] = h;
      if (MODE == TC_BF16X3) lo[o] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
  }
}

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

constexpr uint32_t CB_THREADS = 256;

// a block's sums of a and b into partials[2 block], [2 block + 1]: per thread and per warp in FP32, per block in FP64
// (a sweep's stopping test needs no more, and FP64 per element would cost more than the sweep's memory traffic)
__device__ __forceinline__ void block_sum2f(float a, float b, double* partials) {
  __shared__ double sa[32], sb[32];
  for (int o = 16; o > 0; o >>= 1) { a += __shfl_down_sync(0xffffffffu, a, o); b += __shfl_down_sync(0xffffffffu, b, o); }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (l == 0) { sa[w] = double(a); sb[w] = double(b); }
  __syncthreads();
  if (w == 0) {
    double x = l < nw ? sa[l] : 0.0, y = l < nw ? sb[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) { x += __shfl_down_sync(0xffffffffu, x, o); y += __shfl_down_sync(0xffffffffu, y, o); }
    if (l == 0) { partials[2 * blockIdx.x] = x; partials[2 * blockIdx.x + 1] = y; }
  }
}

// thread per (row, column < R); splits summed in order s = 0, 1, ... (deterministic)
__global__ void __launch_bounds__(CB_THREADS) combine_sweep_kernel(const float* __restrict__ P, uint32_t splits, uint32_t n, uint32_t R,
                                                                   const float* __restrict__ rho, const float* __restrict__ rhs,
                                                                   const float* __restrict__ Xin, float* __restrict__ Y,
                                                                   const float* __restrict__ rs, const float* __restrict__ cs,
                                                                   double* __restrict__ parts) {
  const size_t idx = size_t(blockIdx.x) * CB_THREADS + threadIdx.x;
  float d2 = 0.0f, y2 = 0.0f;
  if (idx < size_t(n) * R) {
    const uint32_t i = uint32_t(idx / R), c = uint32_t(idx % R);
    float acc = 0.0f;
    for (uint32_t s = 0; s < splits; s++) acc += P[(size_t(s) * n + i) * 64 + c];
    if (rs) acc *= rs[i] * cs[c];
    const float y = fmaf(rho[i], acc, rhs[idx]);
    Y[idx] = y;
    const float dd = y - Xin[idx];
    d2 = dd * dd;
    y2 = y * y;
  }
  block_sum2f(d2, y2, parts);
}

__global__ void __launch_bounds__(CB_THREADS) combine_residual_kernel(const float* __restrict__ P, uint32_t splits, uint32_t n, uint32_t R,
                                                                      const float* __restrict__ rho, const float* __restrict__ E,
                                                                      const float* __restrict__ B, float* __restrict__ r,
                                                                      double* __restrict__ parts) {
  const size_t idx = size_t(blockIdx.x) * CB_THREADS + threadIdx.x;
  double r2 = 0.0, b2 = 0.0;
  if (idx < size_t(n) * R) {
    const uint32_t i = uint32_t(idx / R), c = uint32_t(idx % R);
    float acc = 0.0f;
    for (uint32_t s = 0; s < splits; s++) acc += P[(size_t(s) * n + i) * 64 + c];
    const double rr = double(E[idx]) + double(rho[i]) * double(acc) - double(B[idx]);
    r[idx] = float(rr);
    r2 = rr * rr;
    b2 = double(B[idx]) * double(B[idx]);
  }
  block_sum2(r2, b2, parts);
}

__global__ void axpy_kernel(float* __restrict__ B, const float* __restrict__ d, size_t count) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += size_t(gridDim.x) * blockDim.x) B[i] += d[i];
}

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                              const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                              CUtensorMapFloatOOBfill);
EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  });
  return fn;
}

}  // namespace

static_assert(sizeof(CUtensorMap) == sizeof(TcMap), "tensor map size");

bool tc_encode(TcMap* map, const void* base, uint32_t inner, uint32_t rows, uint32_t elt_bytes, uint32_t box_rows, int* code) {
  EncodeFn fn = encode_fn();
  if (!fn) { if (code) *code = -1; return false; }
  const cuuint64_t dims[2] = {inner, rows};
  const cuuint64_t strides[1] = {cuuint64_t(inner) * elt_bytes};
  const cuuint32_t box[2] = {128u / elt_bytes, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(reinterpret_cast<CUtensorMap*>(map), elt_bytes == 2 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 2,
                        const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (code) *code = int(r);
  return r == CUDA_SUCCESS;
}

uint32_t tc_k_elems(int mode) { return mode == TC_FP8 ? 128u : 64u; }

void tc_gemm(int mode, const TcMap* A, const TcMap* A2, const TcMap* B, const TcMap* B2, uint32_t n, uint32_t splits, uint32_t k_tiles,
             float* partials, uint32_t* err, cudaStream_t st) {
  if (mode == TC_BF16) launch_gemm<TC_BF16, 6>(A, A2, B, B2, n, splits, k_tiles, partials, err, st);
  else if (mode == TC_BF16X3) launch_gemm<TC_BF16X3, 4>(A, A2, B, B2, n, splits, k_tiles, partials, err, st);
  else launch_gemm<TC_FP8, 6>(A, A2, B, B2, n, splits, k_tiles, partials, err, st);
}

void tc_split_bf16(const float* F, uint16_t* hi, uint16_t* lo, size_t count, cudaStream_t st) {
  split_bf16_kernel<<<1216, 256, 0, st>>>(F, reinterpret_cast<__nv_bfloat16*>(hi), reinterpret_cast<__nv_bfloat16*>(lo), count);
}

void tc_quant_rows_fp8(const float* F, uint8_t* q, float* row_scale, uint32_t n, cudaStream_t st) {
  quant_rows_fp8_kernel<<<n, 256, 0, st>>>(F, q, row_scale, n);
}

void tc_pack_b(int mode, const float* X, uint32_t n, uint32_t R, uint16_t* hi, uint16_t* lo, uint8_t* q8, float* col_scale,
               uint32_t* col_max, cudaStream_t st) {
  const dim3 grid((n + 31) / 32, 2), block(32, 8);
  if (mode == TC_FP8) {
    cudaMemsetAsync(col_max, 0, 64 * sizeof(uint32_t), st);
    col_max_kernel<<<304, 256, 0, st>>>(X, n, R, col_max);
    pack_b_kernel<TC_FP8><<<grid, block, 0, st>>>(X, n, R, nullptr, nullptr, q8, col_max, col_scale);
  } else if (mode == TC_BF16X3) {
    pack_b_kernel<TC_BF16X3><<<grid, block, 0, st>>>(X, n, R, reinterpret_cast<__nv_bfloat16*>(hi), reinterpret_cast<__nv_bfloat16*>(lo),
                                                     nullptr, nullptr, nullptr);
  } else {
    pack_b_kernel<TC_BF16><<<grid, block, 0, st>>>(X, n, R, reinterpret_cast<__nv_bfloat16*>(hi), nullptr, nullptr, nullptr, nullptr);
  }
}

void tc_combine_sweep(const float* partials, uint32_t splits, uint32_t n, uint32_t R, const float* rho, const float* rhs, const float* Xin,
                      float* Y, const float* row_scale, const float* col_scale, double* norm_partials, uint32_t* n_partials, cudaStream_t st) {
  const uint32_t blocks = uint32_t((size_t(n) * R + CB_THREADS - 1) / CB_THREADS);
  *n_partials = blocks;
  combine_sweep_kernel<<<blocks, CB_THREADS, 0, st>>>(partials, splits, n, R, rho, rhs, Xin, Y, row_scale, col_scale, norm_partials);
}

void tc_combine_residual(const float* partials, uint32_t splits, uint32_t n, uint32_t R, const float* rho, const float* E, const float* B,
                         float* r, double* norm_partials, uint32_t* n_partials, cudaStream_t st) {
  const uint32_t blocks = uint32_t((size_t(n) * R + CB_THREADS - 1) / CB_THREADS);
  *n_partials = blocks;
  combine_residual_kernel<<<blocks, CB_THREADS, 0, st>>>(partials, splits, n, R, rho, E, B, r, norm_partials);
}

void tc_axpy(float* B, const float* d, size_t count, cudaStream_t st) { axpy_kernel<<<1216, 256, 0, st>>>(B, d, count); }

}  // namespace vtk

// ------------------------------------------------------------------------------------------------ wait check
// The bounded-wait path of the pipelines above, exercised on purpose: one block waits on an mbarrier phase that
// completes only if `arrive` is set (one arrival of the barrier's count of 1). Without it the wait runs out after
// `cycles`, sets the error word and the kernel returns: the host sees a timeout and the context stays usable.
namespace vtk {
__global__ void wait_check_kernel(uint64_t cycles, uint32_t arrive, uint32_t* err) {
  __shared__ __align__(8) uint64_t bar;
  const uint32_t b = async::smem_u32(&bar);
  if (threadIdx.x == 0) {
    async::mbar_init(b, 1);
    async::mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && arrive) async::mbar_arrive(b);
  if (threadIdx.x == 0) async::mbar_wait(b, 0, err, cycles);
}
void launch_wait_check(uint64_t cycles, uint32_t arrive, uint32_t* err, cudaStream_t st) {
  wait_check_kernel<<<1, 32, 0, st>>>(cycles, arrive, err);
}
}  // namespace vtk
