// k_project.cu -- projection of a radiance tile onto the SH basis
// (shaders/sh.comp:23-42 for a sample set shared by all probes) and the
// reconstruction of shaders/sh_sum.comp:35-52.
//
// Tile layout: row r = probe*3 + channel, S samples contiguous per row (a
// BF16 tile of hi/lo pairs holds 2S per row: S high parts, then S low parts;
// the sample is their sum).  The basis table is S x 16 FP32 with the sample weight folded in.  One thread
// owns one row; a CTA stages a [128 rows x 64 samples] block of the tile in
// shared memory with coalesced row-segment copies (cp.async for FP32, so a
// thread's copies are all in flight at once; rows padded to 65 words so the
// per-thread column walk is bank-conflict free), and the matching 64 x 16
// basis block is read as warp-wide broadcasts.  Each row's sum runs in FP32
// over its samples in a fixed order, so the result does not depend on the
// launch shape or on other probes in the tile.
#include <cuda_bf16.h>

#include <algorithm>

#include "vlb_device.cuh"
#include "vlb_internal.h"

namespace vlbk {

constexpr int kProjRows = 128;
constexpr int kProjCols = 64;

template <typename T>
__device__ __forceinline__ float to_f32(T v);
template <>
__device__ __forceinline__ float to_f32<float>(float v) { return v; }
template <>
__device__ __forceinline__ float to_f32<uint16_t>(uint16_t v) { return __uint_as_float(uint32_t(v) << 16); }

// Global -> shared copies without a register round trip; valid == false
// writes zeros (no bytes are read from src, which stays a valid address).
__device__ __forceinline__ void cp_async4(float* sdst, const float* gsrc, bool valid) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(sdst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(gsrc), "r"(valid ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async16(float* sdst, const float* gsrc, bool valid) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(sdst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(gsrc), "r"(valid ? 16 : 0) : "memory");
}

// One stage: the [kProjRows x kProjCols] tile block (rows padded to
// kProjCols + 1 words) and the matching basis rows.
constexpr int kProjTileWords = kProjRows * (kProjCols + 1);
constexpr int kProjStageWords = kProjTileWords + kProjCols * 16;
static_assert(kProjTileWords % 4 == 0, "basis block must stay 16-byte aligned");

// Stage loads.  FP32: asynchronous copies, so that all of a thread's loads
// are in flight at once, zero-filled outside the tile; BF16: loads converted
// through registers.  Coalesced: each warp loads 32 rows, 32-sample segments
// per row.
template <typename T>
__device__ __forceinline__ void project_stage(const T* __restrict__ rad, uint32_t rows, uint32_t S, uint32_t s_end,
                                              const float* __restrict__ basis16, uint32_t row0, uint32_t s0,
                                              float* stage, uint32_t split) {
  float(*tile)[kProjCols + 1] = reinterpret_cast<float(*)[kProjCols + 1]>(stage);
  float(*bas)[16] = reinterpret_cast<float(*)[16]>(stage + kProjTileWords);
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t ns = min(uint32_t(kProjCols), s_end - s0);
  if constexpr (sizeof(T) == 4) {
#pragma unroll 8
    for (uint32_t rr = warp; rr < kProjRows; rr += kProjRows / 32) {
      const uint32_t gr = row0 + rr;
#pragma unroll
      for (int h = 0; h < kProjCols / 32; ++h) {
        const uint32_t c = h * 32 + lane;
        const bool ok = gr < rows && c < ns;
        cp_async4(&tile[rr][c], ok ? reinterpret_cast<const float*>(rad) + size_t(gr) * S + s0 + c
                                   : reinterpret_cast<const float*>(rad), ok);
      }
    }
    for (uint32_t i = tid; i < kProjCols * 4; i += kProjRows) {
      const uint32_t j = i / 4, q = i % 4;
      cp_async16(&bas[j][4 * q], j < ns ? basis16 + size_t(s0 + j) * 16 + 4 * q : basis16, j < ns);
    }
  } else {
    for (uint32_t rr = warp; rr < kProjRows; rr += kProjRows / 32) {
      const uint32_t gr = row0 + rr;
#pragma unroll
      for (int h = 0; h < kProjCols / 32; ++h) {
        const uint32_t c = h * 32 + lane;
        float v = 0.f;
        if (gr < rows && c < ns) {
          if (split) {  // hi/lo pair: [rows][2S]
            const size_t r0 = size_t(gr) * 2 * S;
            v = to_f32<T>(rad[r0 + s0 + c]) + to_f32<T>(rad[r0 + S + s0 + c]);
          } else {
            v = to_f32<T>(rad[size_t(gr) * S + s0 + c]);
          }
        }
        tile[rr][c] = v;
      }
    }
    for (uint32_t i = tid; i < kProjCols * 16; i += kProjRows) {
      const uint32_t j = i / 16, k = i % 16;
      bas[j][k] = (j < ns) ? basis16[size_t(s0 + j) * 16 + k] : 0.f;
    }
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// Launch grid: row tiles x sample splits.  A tile of few rows and many
// samples (the reference's 343 probes x 3.14 M samples: 9 row tiles) is split
// along the samples so that about kProjSplitCtas CTAs run; each split sums its
// range in FP32 in order and k_project_reduce adds the splits in FP64 in
// split order.  The split count depends on the tile's shape only, so results
// stay deterministic; tiles with enough rows (C1, C2) run unsplit, one
// sequential FP32 sum per row.
constexpr uint32_t kProjSplitCtas = 304;
constexpr uint32_t kProjMinSplitSamples = 16 * kProjCols;

static uint32_t project_splits(uint32_t rows, uint32_t S, uint32_t* per) {
  const uint32_t tiles = (rows + kProjRows - 1) / kProjRows;
  uint32_t splits = 1;
  if (tiles && tiles < kProjSplitCtas)
    splits = std::max(1u, std::min((kProjSplitCtas + tiles - 1) / tiles, S / kProjMinSplitSamples));
  uint32_t p = (S + splits - 1) / splits;
  p = (p + kProjCols - 1) / kProjCols * kProjCols;  // whole stages
  *per = p;
  return p ? (S + p - 1) / p : 1;
}

size_t project_partial_bytes(uint32_t nprobes, uint32_t S, uint32_t K) {
  uint32_t per;
  const uint32_t splits = project_splits(nprobes * 3, S, &per);
  return splits > 1 ? size_t(splits) * nprobes * 3 * K * sizeof(float) : 0;
}

template <typename T, int K>
__global__ void __launch_bounds__(kProjRows) k_project(const T* __restrict__ rad, uint32_t rows, uint32_t S,
                                                       uint32_t per, const float* __restrict__ basis16,
                                                       float* __restrict__ out, float* __restrict__ partial,
                                                       uint32_t split) {
  __shared__ __align__(16) float stage[kProjStageWords];
  const float(*tile)[kProjCols + 1] = reinterpret_cast<const float(*)[kProjCols + 1]>(stage);
  const float(*bas)[16] = reinterpret_cast<const float(*)[16]>(stage + kProjTileWords);
  const uint32_t tid = threadIdx.x;
  const uint32_t row0 = blockIdx.x * kProjRows;
  const uint32_t row = row0 + tid;
  const uint32_t s_begin = blockIdx.y * per, s_end = min(S, s_begin + per);
  float acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.f;

  for (uint32_t s0 = s_begin; s0 < s_end; s0 += kProjCols) {
    project_stage<T>(rad, rows, S, s_end, basis16, row0, s0, stage, split);
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
#pragma unroll 4
    for (uint32_t j = 0; j < kProjCols; ++j) {
      const float r = tile[tid][j];
      const float4* b4 = reinterpret_cast<const float4*>(bas[j]);
#pragma unroll
      for (int q = 0; q < (K + 3) / 4; ++q) {
        const float4 b = b4[q];
        if (4 * q + 0 < K) acc[4 * q + 0] = fmaf(r, b.x, acc[4 * q + 0]);
        if (4 * q + 1 < K) acc[4 * q + 1] = fmaf(r, b.y, acc[4 * q + 1]);
        if (4 * q + 2 < K) acc[4 * q + 2] = fmaf(r, b.z, acc[4 * q + 2]);
        if (4 * q + 3 < K) acc[4 * q + 3] = fmaf(r, b.w, acc[4 * q + 3]);
      }
    }
    __syncthreads();
  }
  if (row >= rows) return;
  if (gridDim.y == 1) {
    const uint32_t p = row / 3, c = row - 3 * p;
#pragma unroll
    for (int k = 0; k < K; ++k) out[(size_t(p) * K + k) * 3 + c] = acc[k];
  } else {
#pragma unroll
    for (int k = 0; k < K; ++k) partial[(size_t(blockIdx.y) * rows + row) * K + k] = acc[k];
  }
}

// out (probe, k, channel) = the splits' partials of (row, k) added in FP64 in split order.
__global__ void k_project_reduce(const float* __restrict__ partial, uint32_t splits, uint32_t rows, uint32_t K,
                                 float* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * K) return;
  const uint32_t row = i / K, k = i - row * K;
  double sum = 0.0;
  for (uint32_t y = 0; y < splits; ++y) sum += double(partial[(size_t(y) * rows + row) * K + k]);
  const uint32_t p = row / 3, c = row - 3 * p;
  out[(size_t(p) * K + k) * 3 + c] = float(sum);
}

template <typename T>
static void launch_project(const T* rad, uint32_t nprobes, uint32_t S, const float* basis16, uint32_t K, float* out,
                           float* partial, uint32_t split, cudaStream_t s) {
  const uint32_t rows = nprobes * 3;
  const uint32_t tiles = (rows + kProjRows - 1) / kProjRows;
  if (tiles == 0) return;
  uint32_t per = 0;
  const uint32_t splits = S ? project_splits(rows, S, &per) : 1;
  if (!S) per = 0;
  const dim3 grid(tiles, splits);
  if (K == 9) k_project<T, 9><<<grid, kProjRows, 0, s>>>(rad, rows, S, per, basis16, out, partial, split);
  else k_project<T, 16><<<grid, kProjRows, 0, s>>>(rad, rows, S, per, basis16, out, partial, split);
  if (splits > 1) k_project_reduce<<<(rows * K + 255) / 256, 256, 0, s>>>(partial, splits, rows, K, out);
}

void launch_project_f32(const float* radiance, uint32_t nprobes, uint32_t S, const float* basis16, uint32_t K,
                        float* out, float* partial, cudaStream_t s, int* err, int num_sms, uint32_t hold,
                        uint32_t wait_polls) {
  // unsplit tiles (enough rows for the whole GPU) go through the TMA-staged kernel
  uint32_t per = 0;
  const uint32_t rows = nprobes * 3;
  if (err && num_sms && S && project_splits(rows, S, &per) == 1 &&
      launch_project_f32_tma(radiance, nprobes, S, basis16, K, out, err, num_sms, s, hold, wait_polls))
    return;
  launch_project<float>(radiance, nprobes, S, basis16, K, out, partial, 0, s);
}

void launch_project_bf16_simt(const uint16_t* radiance, uint32_t nprobes, uint32_t S, const float* basis16,
                              uint32_t K, float* out, float* partial, uint32_t split, cudaStream_t s) {
  launch_project<uint16_t>(radiance, nprobes, S, basis16, K, out, partial, split, s);
}

// sh_sum.comp:35-52 -- one thread per pixel, direction from the per-column
// (cos phi, sin phi) and per-row (sin theta, cos theta) tables.
template <int K>
__global__ void k_sh_eval_envmap(const float* __restrict__ coeffs, uint32_t w, uint32_t h, float scale,
                                 const float2* __restrict__ col, const float4* __restrict__ rowt, float* __restrict__ out) {
  __shared__ float c[3 * K];
  if (threadIdx.x < 3 * K) c[threadIdx.x] = coeffs[threadIdx.x];
  __syncthreads();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w * h) return;
  const uint32_t y = i / w, x = i - y * w;
  const float2 cs = col[x];
  const float4 rw = rowt[y];
  float Y[K];
  sh_basis<(K == 9 ? 2 : 3)>(rw.x * cs.x, rw.x * cs.y, rw.y, Y);
  float r = 0.f, g = 0.f, b = 0.f;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    r = fmaf(c[3 * k], Y[k], r);
    g = fmaf(c[3 * k + 1], Y[k], g);
    b = fmaf(c[3 * k + 2], Y[k], b);
  }
  out[3 * size_t(i)] = scale * r;
  out[3 * size_t(i) + 1] = scale * g;
  out[3 * size_t(i) + 2] = scale * b;
}

void launch_sh_eval_envmap(const float* coeffs, uint32_t K, uint32_t w, uint32_t h, float scale, const float2* col_tab,
                           const float4* row_tab, float* out, cudaStream_t s) {
  const uint32_t n = w * h;
  if (n == 0) return;
  const uint32_t grid = (n + 255) / 256;
  if (K == 9) k_sh_eval_envmap<9><<<grid, 256, 0, s>>>(coeffs, w, h, scale, col_tab, row_tab, out);
  else k_sh_eval_envmap<16><<<grid, 256, 0, s>>>(coeffs, w, h, scale, col_tab, row_tab, out);
}

// Sky SH evaluated along directions: shaders/skybox_sh.rmiss:14-25 with the
// coefficient count fixed to K (the reference sums 16 bands, 256 terms, over a
// 16-coefficient buffer).
template <int LMAX>
__global__ void k_sh_eval_dirs(const float* __restrict__ coeffs, const float* __restrict__ dirs, uint32_t n,
                               float* __restrict__ out) {
  constexpr int K = sh_k<LMAX>();
  __shared__ float c[3 * K];
  if (threadIdx.x < 3 * K) c[threadIdx.x] = coeffs[threadIdx.x];
  __syncthreads();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x = dirs[3 * size_t(i)], y = dirs[3 * size_t(i) + 1], z = dirs[3 * size_t(i) + 2];
  const float rn = rsqrtf(x * x + y * y + z * z);
  x *= rn; y *= rn; z *= rn;
  float Y[16];
  sh_basis<LMAX>(x, y, z, Y);
  float r = 0.f, g = 0.f, b = 0.f;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    r = fmaf(c[3 * k], Y[k], r);
    g = fmaf(c[3 * k + 1], Y[k], g);
    b = fmaf(c[3 * k + 2], Y[k], b);
  }
  out[3 * size_t(i)] = r;
  out[3 * size_t(i) + 1] = g;
  out[3 * size_t(i) + 2] = b;
}

void launch_sh_eval_dirs(const float* coeffs, uint32_t lmax, const float* dirs, uint32_t n, float* out,
                         cudaStream_t s) {
  if (n == 0) return;
  const uint32_t grid = (n + 255) / 256;
  if (lmax == 3) k_sh_eval_dirs<3><<<grid, 256, 0, s>>>(coeffs, dirs, n, out);
  else k_sh_eval_dirs<2><<<grid, 256, 0, s>>>(coeffs, dirs, n, out);
}

}  // namespace vlbk

namespace vlbk {

// The reference's carry-over accumulator (vlb_bake VLB_BAKE_REF_ACCUMULATE):
// out[p][v] <- sum of out[q][v] over q <= p, in FP64, rounded once.  One CTA
// per value v walks the probes in chunks of 256: a block-wide inclusive scan
// of the chunk plus the running carry of the chunks before it (a fixed order).
__global__ void __launch_bounds__(256) k_probe_prefix(float* __restrict__ out, uint32_t nprobes, uint32_t V) {
  __shared__ double wsum[8];
  const uint32_t v = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double carry = 0.0;
  for (uint32_t p0 = 0; p0 < nprobes; p0 += 256) {
    const uint32_t p = p0 + tid;
    double x = p < nprobes ? double(out[size_t(p) * V + v]) : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, x, o);
      if (int(lane) >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    double before = carry;
    for (uint32_t k = 0; k < warp; ++k) before += wsum[k];
    double total = carry;
    for (uint32_t k = 0; k < 8; ++k) total += wsum[k];
    if (p < nprobes) out[size_t(p) * V + v] = float(before + x);
    __syncthreads();
    carry = total;
  }
}

void launch_probe_prefix(float* out, uint32_t nprobes, uint32_t V, cudaStream_t s) {
  if (nprobes && V) k_probe_prefix<<<V, 256, 0, s>>>(out, nprobes, V);
}

}  // namespace vlbk
