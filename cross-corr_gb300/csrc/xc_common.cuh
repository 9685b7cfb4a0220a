// xc_common.cuh -- shared host/device helpers of the GB300 cross-correlation
// library: status plumbing, TMA tensor maps, mbarrier PTX wrappers.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "xcorr.h"

namespace xc {

// ---------------------------------------------------------------------------
// Error reporting: every C-ABI call returns an xc_status and records a
// thread-local message; no exception crosses the ABI.
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
xc_status fail(xc_status st, const std::string& msg);
xc_status from_cuda(cudaError_t err, const char* what);

#define XC_CUDA_TRY(expr)                                   \
  do {                                                      \
    cudaError_t e__ = (expr);                               \
    if (e__ != cudaSuccess) return ::xc::from_cuda(e__, #expr); \
  } while (0)

#define XC_TRY(expr)                      \
  do {                                    \
    xc_status s__ = (expr);               \
    if (s__ != XC_OK) return s__;         \
  } while (0)

inline int div_up(long a, long b) { return (int)((a + b - 1) / b); }

// ---------------------------------------------------------------------------
// TMA tensor maps.  cuTensorMapEncodeTiled is fetched through the runtime's
// driver entry point so the library does not link libcuda directly.
// ---------------------------------------------------------------------------
// Encodes a tiled, non-swizzled tensor map with zero fill for out-of-bounds
// reads.  dims/strides are innermost first; strides[i] is the byte stride of
// dimension i+1 (strides of dims 1..rank-1).  Returns false (and sets the
// error message) when the driver rejects the description.
bool encode_tiled(CUtensorMap* map, CUtensorMapDataType dtype, int rank, const void* base, const uint64_t* dims,
                  const uint64_t* byte_strides, const uint32_t* box, CUtensorMapSwizzle swizzle);

// Device-side error flag used by bounded waits: a kernel whose wait runs out
// records a code here and returns instead of hanging.
struct DeviceFlags {
  unsigned int timeout;  // non-zero when some bounded wait expired
  unsigned int where;    // kernel-specific code of the first expiry
};
DeviceFlags* device_flags();  // per-device address of a __device__ variable (no allocation)
unsigned long long current_context_id();  // unique ID of the current CUDA context, 0 if unknown
xc_status check_device_flags(cudaStream_t stream);

#if defined(__CUDACC__)
// ---------------------------------------------------------------------------
// PTX wrappers (sm_90+; used by the sm_103a kernels).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_count(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Arrives on `bar` once all cp.async copies this thread issued so far have
// landed (without raising the barrier's expected count).
__device__ __forceinline__ void cp_async_mbar_arrive(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// try_wait with a suspend-time hint: a waiting thread sleeps (no issue
// slots) until the phase completes or about `ns` nanoseconds pass.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase.  Returns false when the iteration budget
// (each try_wait already suspends for a hardware-chosen interval) runs out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_iters = (1u << 22)) {
  for (uint32_t i = 0; i < max_iters; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  return false;
}

__device__ __forceinline__ void record_timeout(DeviceFlags* flags, unsigned int where) {
  if (flags != nullptr) {
    if (atomicCAS(&flags->timeout, 0u, 1u) == 0u) flags->where = where;
  }
}

// 2D..5D tiled TMA loads into shared memory, completing on an mbarrier.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cta.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cta.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6}], "
      "[%2];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}

// cp.async with zero fill: copies `bytes` (4, 8 or 16) when `valid`, else
// writes zeros.  Used by the loaders for row pitches TMA cannot describe.
template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void* dst, const void* src, bool valid) {
  const uint32_t n = valid ? BYTES : 0u;
  if constexpr (BYTES == 16) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(n) : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(smem_u32(dst)), "l"(src), "n"(BYTES), "r"(n)
                 : "memory");
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
#endif  // __CUDACC__

}  // namespace xc
