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

// ---- FP32 tile projection through TMA (the default path's projection) -------------
// The same per-row sums as k_project<float> (one thread a row, every sample in
// order, FP32 fmaf: the same bits), with the tile staged by the TMA engine:
// a producer warp streams [256 rows x 32 samples] boxes of the row-major tile
// (128-byte rows, 128-byte swizzle) and the matching 32 x 16 basis rows (a 1-D
// bulk copy) into a kF32Stages ring; four consumer warps, two rows a thread
// (t and t + 128: each basis broadcast serves both), read their rows' 16-byte
// chunks at the swizzled positions (chunk q of row r sits at q ^ (r & 7):
// eight consecutive rows hit eight different bank groups, no conflicts).
// Persistent CTAs take row tiles in turn.  A two-stage ring keeps three CTAs
// (twelve consumer warps) on an SM: measured on the tile [786,432 x
// 1024] at 92 % of the HBM copy rate (three stages, two CTAs: 74 %; one row a
// thread: 49 %; the cp.async kernel k_project<float>: 62 %).
constexpr int kF32Rows = 256, kF32Cols = 32;  // two rows a consumer thread: t and t + 128
constexpr int kF32Stages = 2;
constexpr int kF32Threads = 160;                                     // 4 consumer warps + 1 producer warp
constexpr uint32_t kF32TileBytes = kF32Rows * kF32Cols * 4;         // 32 KiB
constexpr uint32_t kF32BasBytes = kF32Cols * 16 * 4;                // 2 KiB
constexpr uint32_t kF32StageBytes = kF32TileBytes + kF32BasBytes;   // 34 KiB, a multiple of 1024
constexpr size_t kF32SmemBytes = size_t(kF32Stages) * kF32StageBytes + 1024;
static_assert(kF32StageBytes % 1024 == 0, "stages stay 1024-byte aligned for the swizzle");

template <int K>
__global__ void __launch_bounds__(kF32Threads) k_project_f32_tma(const __grid_constant__ CUtensorMap tm,
                                                                 const float* __restrict__ basis16, uint32_t rows,
                                                                 uint32_t S, float* __restrict__ out, int* err,
                                                                 uint32_t hold, uint32_t polls) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full[kF32Stages], empty[kF32Stages];
  __shared__ volatile int abort_flag;
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint8_t* base = smem_raw + (((smem_u32(smem_raw) + 1023u) & ~1023u) - smem_u32(smem_raw));
  const uint32_t ntiles = (rows + kF32Rows - 1) / kF32Rows;
  const uint32_t nst = (S + kF32Cols - 1) / kF32Cols;
  if (tid == 0) {
    for (int i = 0; i < kF32Stages; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], 4); }
    abort_flag = 0;
    fence_mbar_init();
  }
  __syncthreads();

  if (warp == 4) {  // producer
    if (lane == 0 && !hold) {  // hold (a test hook): no copy is issued, the consumers' waits give up
      uint32_t seq = 0;
      for (uint32_t tile = blockIdx.x; tile < ntiles && !abort_flag; tile += gridDim.x)
        for (uint32_t c = 0; c < nst; ++c, ++seq) {
          const uint32_t st = seq % kF32Stages;
          if (!mbar_wait_bounded(&empty[st], ((seq / kF32Stages) & 1u) ^ 1u, err, polls)) { abort_flag = 1; break; }
          const uint32_t nt = min(uint32_t(kF32Cols), S - c * kF32Cols);
          uint8_t* sb = base + size_t(st) * kF32StageBytes;
          mbar_arrive_expect_tx(&full[st], kF32TileBytes + nt * 64);
          tma_load_2d(sb, &tm, int(c * kF32Cols), int(tile * kF32Rows), &full[st]);
          bulk_g2s(sb + kF32TileBytes, basis16 + size_t(c) * kF32Cols * 16, nt * 64, &full[st]);
        }
      // copies still in flight land before the CTA may exit
      const uint32_t first = seq > uint32_t(kF32Stages) ? seq - kF32Stages : 0;
      for (uint32_t q = first; q < seq; ++q)
        mbar_wait_bounded(&full[q % kF32Stages], (q / kF32Stages) & 1u, err, 1u << 16);
    }
    return;
  }

  constexpr int NQ = (K + 3) / 4;  // basis float4 per sample
  uint32_t seq = 0;
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    float acc[2][K];  // rows t and t + 128 of the tile
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int k = 0; k < K; ++k) acc[h][k] = 0.f;
    for (uint32_t c = 0; c < nst; ++c, ++seq) {
      const uint32_t st = seq % kF32Stages;
      if (!mbar_wait_bounded(&full[st], (seq / kF32Stages) & 1u, err, polls)) abort_flag = 1;
      if (abort_flag) break;
      const uint8_t* sb = base + size_t(st) * kF32StageBytes;
      const float4* bas = reinterpret_cast<const float4*>(sb + kF32TileBytes);  // [32][16] floats
      // the last stage of a row may be partial: its basis rows past nt were not copied
      const uint32_t nt = min(uint32_t(kF32Cols), S - c * kF32Cols);
#pragma unroll
      for (int q = 0; q < kF32Cols / 4; ++q) {
        // rows t and t + 128: the same swizzle phase (t & 7)
        const uint32_t off = ((q ^ (tid & 7)) << 4);
        const float4 v0 = *reinterpret_cast<const float4*>(sb + tid * 128 + off);
        const float4 v1 = *reinterpret_cast<const float4*>(sb + (tid + 128) * 128 + off);
        const float r4[2][4] = {{v0.x, v0.y, v0.z, v0.w}, {v1.x, v1.y, v1.z, v1.w}};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (uint32_t(4 * q + e) >= nt) break;
          const float4* b4 = bas + (4 * q + e) * 4;
#pragma unroll
          for (int g = 0; g < NQ; ++g) {
            const float4 b = b4[g];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              if (4 * g + 0 < K) acc[h][4 * g + 0] = fmaf(r4[h][e], b.x, acc[h][4 * g + 0]);
              if (4 * g + 1 < K) acc[h][4 * g + 1] = fmaf(r4[h][e], b.y, acc[h][4 * g + 1]);
              if (4 * g + 2 < K) acc[h][4 * g + 2] = fmaf(r4[h][e], b.z, acc[h][4 * g + 2]);
              if (4 * g + 3 < K) acc[h][4 * g + 3] = fmaf(r4[h][e], b.w, acc[h][4 * g + 3]);
            }
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[st]);  // this warp is done with the stage
    }
    if (abort_flag) break;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t row = tile * kF32Rows + tid + 128 * h;
      if (row < rows) {
        const uint32_t p = row / 3, ch = row - 3 * p;
#pragma unroll
        for (int k = 0; k < K; ++k) out[(size_t(p) * K + k) * 3 + ch] = acc[h][k];
      }
    }
  }
}

bool make_map_f32(CUtensorMap* m, const void* ptr, uint64_t S, uint64_t rows) {
  EncodeTiled fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {S, rows};
  const cuuint64_t strides[1] = {S * 4};
  const cuuint32_t box[2] = {uint32_t(kF32Cols), uint32_t(kF32Rows)};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(ptr), dims, strides, box, estr,
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

namespace vlbk {

int launch_project_f32_tma(const float* radiance, uint32_t nprobes, uint32_t S, const float* basis16, uint32_t K,
                           float* out, int* err, int num_sms, cudaStream_t s, uint32_t hold, uint32_t wait_polls) {
  const uint32_t rows = nprobes * 3;
  // small tiles (fewer 256-row tiles than SMs) stay with the cp.async kernel's
  // 128-row CTAs, which spread them over more SMs
  if (rows == 0 || S == 0 || S % 4 || (reinterpret_cast<uintptr_t>(radiance) % 16) ||
      (reinterpret_cast<uintptr_t>(basis16) % 16) || (rows + kF32Rows - 1) / kF32Rows < uint32_t(num_sms))
    return 0;
  CUtensorMap tm;
  if (!make_map_f32(&tm, radiance, S, rows)) return 0;
  static std::atomic<uint64_t> opted9{0}, opted16{0};
  const uint32_t ntiles = (rows + kF32Rows - 1) / kF32Rows;
  const uint32_t polls = wait_polls ? wait_polls : kWaitPolls;
  if (K == 9) {
    smem_opt_in(k_project_f32_tma<9>, int(kF32SmemBytes), opted9);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_project_f32_tma<9>, kF32Threads, kF32SmemBytes);
    const uint32_t grid = std::min<uint32_t>(ntiles, uint32_t(num_sms) * uint32_t(std::max(per_sm, 1)));
    k_project_f32_tma<9><<<grid, kF32Threads, kF32SmemBytes, s>>>(tm, basis16, rows, S, out, err, hold, polls);
  } else {
    smem_opt_in(k_project_f32_tma<16>, int(kF32SmemBytes), opted16);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_project_f32_tma<16>, kF32Threads, kF32SmemBytes);
    const uint32_t grid = std::min<uint32_t>(ntiles, uint32_t(num_sms) * uint32_t(std::max(per_sm, 1)));
    k_project_f32_tma<16><<<grid, kF32Threads, kF32SmemBytes, s>>>(tm, basis16, rows, S, out, err, hold, polls);
  }
  return 1;
}

}  // namespace vlbk
