// Tensor-core (tcgen05) Jacobi sweeps of the node radiosity with many right-hand sides (vt_tc.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace vtk {

enum TcMode { TC_BF16 = 0, TC_BF16X3 = 1, TC_FP8 = 2 };

// opaque tensor-map storage (CUtensorMap is 128 bytes, 64-byte aligned)
struct alignas(64) TcMap { unsigned char bytes[128]; };

// F (n x n, K contiguous) and the transposed right-hand sides Bt (r x n, K contiguous) as TMA tiles:
// mode BF16 / BF16X3: bf16 elements, boxes of 64 x 128 (F) and 64 x 64 (Bt); FP8: bytes, boxes of 128 x 128 / 128 x 64.
// Returns false (with the driver's error code in *code) when the map cannot be encoded.
bool tc_encode(TcMap* map, const void* base, uint32_t inner, uint32_t rows, uint32_t elt_bytes, uint32_t box_rows, int* code);

// partials[s][i][c] = sum over split s's K range of A[i][k] B[c][k]  (c < 64), three products for BF16X3
void tc_gemm(int mode, const TcMap* A, const TcMap* A2, const TcMap* B, const TcMap* B2, uint32_t n, uint32_t splits, uint32_t k_tiles,
             float* partials, uint32_t* err, cudaStream_t st);
uint32_t tc_k_elems(int mode);   // K elements per pipeline stage (128 bytes of a row)

// F (fp32) -> hi = bf16(F), lo = bf16(F - hi)
void tc_split_bf16(const float* F, uint16_t* hi, uint16_t* lo, size_t count, cudaStream_t st);
// F (fp32, n x n) -> q = e4m3(F / s_i), s_i = max_j |F_ij| / 448 (one scale per row)
void tc_quant_rows_fp8(const float* F, uint8_t* q, float* row_scale, uint32_t n, cudaStream_t st);
// X (n x R fp32, row-major) -> Bt (64 x n, transposed, rows >= R zero): bf16 hi [and lo], or e4m3 with one scale per column
void tc_pack_b(int mode, const float* X, uint32_t n, uint32_t R, uint16_t* hi, uint16_t* lo, uint8_t* q8, float* col_scale,
               uint32_t* col_max, cudaStream_t st);
// Jacobi sweep epilogue: Y = rhs + rho * (sum_s partials) [* s_i t_c], norms of Y - Xin and Y (per block)
void tc_combine_sweep(const float* partials, uint32_t splits, uint32_t n, uint32_t R, const float* rho, const float* rhs, const float* Xin,
                      float* Y, const float* row_scale, const float* col_scale, double* norm_partials, uint32_t* n_partials, cudaStream_t st);
// accurate residual: r = E + rho * acc - B in float64 (stored fp32), norms of r and B (per block)
void tc_combine_residual(const float* partials, uint32_t splits, uint32_t n, uint32_t R, const float* rho, const float* E, const float* B,
                         float* r, double* norm_partials, uint32_t* n_partials, cudaStream_t st);
// B += d
void tc_axpy(float* B, const float* d, size_t count, cudaStream_t st);

// one bounded mbarrier wait that completes only when `arrive` is set; *err is set when it runs out after `cycles`
void launch_wait_check(uint64_t cycles, uint32_t arrive, uint32_t* err, cudaStream_t st);

}  // namespace vtk
