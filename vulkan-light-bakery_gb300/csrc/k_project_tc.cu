// k_project_tc.cu -- SH projection of a BF16 radiance tile on the 5th-generation
// tensor cores (tcgen05), the mixed-precision form of shaders/sh.comp:23-42 for
// a sample set shared by all probes.
//
//   C[row, n] = sum_s A[row, s] * Bt[n, s]      row = probe*3 + channel
//   A  : radiance tile, BF16, [rows][S] (S contiguous)            -- streamed from HBM
//   Bt : weighted basis, BF16, [32][S]: n < 16 the high part, n >= 16 the
//        low part (basis - high) of w_s * Y_k(b_s); the sum of both halves
//        carries ~16 mantissa bits of the basis
//   out[probe][k][channel] = C[row, k] + C[row, 16 + k]
//
// One persistent CTA per SM; its warps have fixed roles:
//   warp 0      TMA producer (one elected lane): tiled bulk-tensor copies of a
//               128 x 64 A tile and the matching 32 x 64 Bt tile into an
//               8-stage ring, 128-byte swizzle, completion on mbarriers
//   warp 1      MMA issuer (one lane): 4 x tcgen05.mma.kind::f16 (M=128, N=32,
//               K=16) per stage into one of two TMEM accumulators (2 x 32 cols)
//   warps 2..5  epilogue: tcgen05.ld of the accumulator rows (warp w reads TMEM
//               lanes 32*(w%4)..+31), hi+lo combine, store
// Every mbarrier wait is bounded; a timeout sets the error counter, stops all
// roles, waits (bounded) for copies in flight and frees TMEM before exit.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "vlb_device.cuh"
#include "vlb_internal.h"

namespace vlbk {
namespace {

constexpr int kTcThreads = 192;  // 6 warps
constexpr int kTileM = 128, kTileN = 32, kTileK = 64;  // K per stage: 64 BF16 = 128 B = one swizzle row
constexpr int kStages = 8;
constexpr uint32_t kStageA = kTileM * kTileK * 2;      // 16 KiB
constexpr uint32_t kStageB = kTileN * kTileK * 2;      // 4 KiB
constexpr uint32_t kStageBytes = kStageA + kStageB;    // 20 KiB, multiple of 1024
constexpr uint32_t kTmemCols = 64;                     // two 32-column accumulators
constexpr size_t kSmemBytes = size_t(kStages) * kStageBytes + 1024;  // + alignment slack

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Shared-memory matrix descriptor: K-major tile, 128-byte swizzle, 8-row
// swizzle atoms 1024 bytes apart (stride byte offset); the leading byte offset
// is not used by swizzled K-major layouts.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= uint64_t((addr >> 4) & 0x3FFFu);
  d |= uint64_t(1) << 16;              // leading byte offset (unused), 16 B
  d |= uint64_t(1024 >> 4) << 32;      // stride byte offset: 1024 B
  d |= uint64_t(1) << 46;              // descriptor version for this architecture
  d |= uint64_t(2) << 61;              // swizzle: 128 B
  return d;
}

// Instruction descriptor for kind::f16: D FP32, A and B BF16, both K-major.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(kTileN >> 3) << 17) |
                            (uint32_t(kTileM >> 4) << 24);

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcShared {
  uint64_t full[kStages];
  uint64_t empty[kStages];
  uint64_t acc_full[2];
  uint64_t acc_empty[2];
  uint32_t tmem_base;
  volatile int abort;  // set by any role whose bounded wait gave up; read by all
};

__global__ void __launch_bounds__(kTcThreads, 1)
    k_project_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, uint32_t rows,
                 uint32_t S, uint32_t K, float* __restrict__ out, int* err, uint32_t hold, uint32_t polls) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ TcShared sh;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  uint8_t* gbase = smem_raw + (base - smem_u32(smem_raw));
  const uint32_t ntiles = (rows + kTileM - 1) / kTileM;
  const uint32_t nkb = (S + kTileK - 1) / kTileK;

  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) { mbar_init(&sh.full[i], 1); mbar_init(&sh.empty[i], 1); }
    for (int i = 0; i < 2; ++i) { mbar_init(&sh.acc_full[i], 1); mbar_init(&sh.acc_empty[i], kTileM); }
    sh.abort = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(&sh.tmem_base, kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sh.tmem_base;

  if (warp == 0) {
    if (lane == 0 && !hold) {  // hold (a test hook): no copy is issued, the waits below give up
      uint32_t issued = 0;
      for (uint32_t tile = blockIdx.x; tile < ntiles && !sh.abort; tile += gridDim.x) {
        for (uint32_t kb = 0; kb < nkb; ++kb, ++issued) {
          const uint32_t st = issued % kStages, round = issued / kStages;
          if (!mbar_wait_bounded(&sh.empty[st], (round & 1u) ^ 1u, err, polls)) { sh.abort = 1; break; }
          mbar_arrive_expect_tx(&sh.full[st], kStageBytes);
          uint8_t* sa = gbase + size_t(st) * kStageBytes;
          tma_load_2d(sa, &tmA, int(kb * kTileK), int(tile * kTileM), &sh.full[st]);
          tma_load_2d(sa + kStageA, &tmB, int(kb * kTileK), 0, &sh.full[st]);
        }
      }
      // copies still in flight land before the CTA may exit
      const uint32_t first = issued > kStages ? issued - kStages : 0;
      for (uint32_t q = first; q < issued; ++q)
        mbar_wait_bounded(&sh.full[q % kStages], (q / kStages) & 1u, err, 1u << 16);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      uint32_t used = 0, it = 0;
      for (uint32_t tile = blockIdx.x; tile < ntiles && !sh.abort; tile += gridDim.x, ++it) {
        const uint32_t acc = it & 1u;
        if (!mbar_wait_bounded(&sh.acc_empty[acc], ((it >> 1) & 1u) ^ 1u, err, polls)) { sh.abort = 1; break; }
        tc_fence_after();
        const uint32_t d = tmem + acc * kTileN;
        for (uint32_t kb = 0; kb < nkb; ++kb, ++used) {
          const uint32_t st = used % kStages;
          if (!mbar_wait_bounded(&sh.full[st], (used / kStages) & 1u, err, polls)) { sh.abort = 1; break; }
          tc_fence_after();
          const uint32_t sa = base + st * kStageBytes, sb = sa + kStageA;
#pragma unroll
          for (int k = 0; k < kTileK / 16; ++k)
            mma_bf16(d, smem_desc(sa + 32 * k), smem_desc(sb + 32 * k), kIdesc, (kb | k) != 0);
          mma_commit(&sh.empty[st]);  // the stage is free once these MMAs have read it
        }
        if (sh.abort) break;
        mma_commit(&sh.acc_full[acc]);
      }
    }
  } else {
    // epilogue warps 2..5: TMEM lanes 32*(warp%4) .. +31
    const uint32_t lane_base = 32u * (warp & 3u);
    uint32_t it = 0;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      const uint32_t acc = it & 1u;
      if (!mbar_wait_bounded(&sh.acc_full[acc], (it >> 1) & 1u, err, polls)) { sh.abort = 1; break; }
      tc_fence_after();
      float v[32];
      tmem_ld32(tmem + (lane_base << 16) + acc * kTileN, v);
      tc_fence_before();
      mbar_arrive(&sh.acc_empty[acc]);
      const uint32_t row = tile * kTileM + lane_base + lane;
      if (row < rows) {
        const uint32_t p = row / 3, c = row - 3 * p;
        float* o = out + size_t(p) * K * 3 + c;
#pragma unroll
        for (uint32_t k = 0; k < 16; ++k)
          if (k < K) o[3 * k] = v[k] + v[16 + k];
      }
      if (sh.abort) break;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  });
  return fn;
}

// 2-D BF16 tensor map: inner extent `inner` (elements, row pitch `pitch`
// elements), `outer` rows, box 64 x box_rows, 128-byte swizzle, zero fill.
bool make_map(CUtensorMap* m, const void* ptr, uint64_t inner, uint64_t outer, uint64_t pitch, uint32_t box_rows) {
  EncodeTiled fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {inner, outer};
  const cuuint64_t strides[1] = {pitch * 2};
  const cuuint32_t box[2] = {uint32_t(kTileK), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool project_tc_supported(const void* radiance, uint32_t S) {
  return S > 0 && S % 8 == 0 && (reinterpret_cast<uintptr_t>(radiance) % 16) == 0 && encode_fn() != nullptr;
}

int launch_project_tc(const uint16_t* radiance, uint32_t nprobes, uint32_t S, const uint16_t* basis_bt,
                      uint32_t bt_pitch, uint32_t K, float* out, int* err, int num_sms, cudaStream_t s,
                      uint32_t hold, uint32_t wait_polls) {
  const uint32_t rows = nprobes * 3;
  if (rows == 0) return 0;
  CUtensorMap ta, tb;
  if (!make_map(&ta, radiance, S, rows, S, kTileM)) return -1;
  if (!make_map(&tb, basis_bt, S, kTileN, bt_pitch, kTileN)) return -1;
  static std::atomic<uint64_t> opted{0};
  smem_opt_in(k_project_tc, int(kSmemBytes), opted);
  const uint32_t ntiles = (rows + kTileM - 1) / kTileM;
  const uint32_t grid = std::min<uint32_t>(ntiles, uint32_t(num_sms));
  k_project_tc<<<grid, kTcThreads, kSmemBytes, s>>>(ta, tb, rows, S, K, out, err, hold,
                                                     wait_polls ? wait_polls : kWaitPolls);
  return 1;
}

}  // namespace vlbk
