// mbarrier and bulk-copy (TMA) helpers shared by the tcgen05 GEMM (vt_tc.cu) and the TMA-fed matvec
// (vt_radiosity.cu). Every wait is bounded by a clock limit: when it runs out the caller's error flag is set and the
// wait returns false, never a hang.
#pragma once

#include <cstdint>

namespace vtk {
namespace async {

constexpr unsigned long long WAIT_CYCLES = 4000000000ull;   // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// bounded wait for the completion of the phase with parity `parity`; false (and *err set) when it runs out
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t* err, unsigned long long limit = WAIT_CYCLES) {
  const unsigned long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n selp.u32 %0, 1, 0, P;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > limit) { atomicOr(err, 1u); return false; }
  }
}
// untiled bulk copy global -> shared, completing on an mbarrier (both addresses 16-byte aligned, bytes % 16 == 0)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
               : "memory");
}

}  // namespace async
}  // namespace vtk
