// vlb_device.cuh -- device helpers shared by the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

namespace vlbk {

// Opts a kernel in to `bytes` of dynamic shared memory on the current device,
// once per device (the attribute is per device; `done` is the caller's
// per-kernel bit set of devices already set).
template <class F>
inline void smem_opt_in(F* kernel, int bytes, std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = dev < 64 ? (1ull << dev) : 0;
  if (bit && (done.load(std::memory_order_relaxed) & bit)) return;
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  done.fetch_or(bit, std::memory_order_relaxed);
}

// Real SH basis with the reference's 6-digit constants
// (shaders/sh_common.h:26-116), index k = l(l+1)+m, l <= LMAX.
template <int LMAX>
__device__ __forceinline__ void sh_basis(float x, float y, float z, float* o) {
  o[0] = 0.282095f;
  o[1] = -0.488603f * y;
  o[2] = 0.488603f * z;
  o[3] = -0.488603f * x;
  o[4] = 1.092548f * x * y;
  o[5] = -1.092548f * y * z;
  o[6] = 0.315392f * (2.0f * z * z - x * x - y * y);
  o[7] = -1.092548f * x * z;
  o[8] = 0.546274f * (x * x - y * y);
  if constexpr (LMAX >= 3) {
    const float x2 = x * x, y2 = y * y, z2 = z * z;
    o[9] = -0.590044f * y * (3.0f * x2 - y2);
    o[10] = 2.890611f * x * y * z;
    o[11] = -0.457046f * y * (4.0f * z2 - x2 - y2);
    o[12] = 0.373176f * z * (2.0f * z2 - 3.0f * x2 - 3.0f * y2);
    o[13] = -0.457046f * x * (4.0f * z2 - x2 - y2);
    o[14] = 1.445306f * z * (x2 - y2);
    o[15] = -0.590044f * x * (x2 - 3.0f * y2);
  }
}

template <int LMAX>
__host__ __device__ constexpr int sh_k() { return (LMAX + 1) * (LMAX + 1); }

// ---- mbarrier + bulk async copy (TMA engine, non-tensor form) ----------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: gives up after max_tries polls (each try_wait may suspend the
// thread for a hardware-defined interval) and bumps the timeout counter.
constexpr uint32_t kWaitPolls = 1u << 22;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* err,
                                                  uint32_t max_tries = kWaitPolls) {
  for (uint32_t i = 0; i < max_tries; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  if (err) atomicAdd(err + 1, 1);
  return false;
}

// 1-D bulk copy global -> shared, completion counted on the mbarrier.
// dst and src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ---- warp helpers -----------------------------------------------------------------
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace vlbk
