// k_lbvh.cu -- device LBVH build, replacing the driver-built BLAS/TLAS of
// Scene_t::buildAS / buildAccelerationStructures (src/scene_manager.cpp:339-442).
//
// Karras 2012 ("Maximizing parallelism in the construction of BVHs, octrees
// and k-d trees").  Every step is either integer arithmetic or an IEEE FP32
// operation with explicit rounding, so the tree is bit-exact with the CPU
// build in the oracle:
//   1. per triangle: FP32 AABB, centroid (lo + hi) * 0.5;
//   2. centroid bounds (min/max reduction);
//   3. 30-bit Morton code from q = (c - lo) * (1024 / extent), clamped;
//   4. stable LSD radix sort of (code, triangle) -- 4 passes of 8 bits;
//   5. Karras split search with ties broken by index (32 + clz(i ^ j));
//   6. bottom-up refit with one atomic counter per internal node (min/max
//      unions are order independent);
//   7. packing into the traversal layout: internal node = 4 float4 holding
//      both children's boxes (widened by a relative 2^-20 so that the box
//      tests are conservative) and references; triangle = 3 float4 (v0 | id,
//      e1, e2) in leaf order.
#include <algorithm>

#include "vlb_device.cuh"
#include "vlb_internal.h"

namespace vlbk {

constexpr int kRsThreads = 256;
constexpr int kRsTile = 4096;  // keys per sort CTA
constexpr int kRedThreads = 256;

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void k_tri_bounds(const float* __restrict__ pos, uint32_t stride, const uint32_t* __restrict__ idx,
                             uint32_t n, float* __restrict__ tb, float* __restrict__ cen) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float p0 = pos[size_t(i0) * stride + a], p1 = pos[size_t(i1) * stride + a], p2 = pos[size_t(i2) * stride + a];
    const float lo = fminf(p0, fminf(p1, p2)), hi = fmaxf(p0, fmaxf(p1, p2));
    tb[6 * size_t(t) + a] = lo;
    tb[6 * size_t(t) + 3 + a] = hi;
    cen[3 * size_t(t) + a] = __fmul_rn(__fadd_rn(lo, hi), 0.5f);
  }
}

__global__ void k_cbounds_partial(const float* __restrict__ cen, uint32_t n, float* __restrict__ part) {
  __shared__ float s[6][kRedThreads];
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float c = cen[3 * size_t(t) + a];
      lo[a] = fminf(lo[a], c);
      hi[a] = fmaxf(hi[a], c);
    }
#pragma unroll
  for (int a = 0; a < 3; ++a) { s[a][threadIdx.x] = lo[a]; s[3 + a][threadIdx.x] = hi[a]; }
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        s[a][threadIdx.x] = fminf(s[a][threadIdx.x], s[a][threadIdx.x + w]);
        s[3 + a][threadIdx.x] = fmaxf(s[3 + a][threadIdx.x], s[3 + a][threadIdx.x + w]);
      }
    __syncthreads();
  }
  if (threadIdx.x < 6) part[6 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

// params: lo[3], scale[3] with scale = 1024 / (hi - lo) (0 for a flat axis)
__global__ void k_cbounds_final(const float* __restrict__ part, uint32_t nblk, float* __restrict__ params) {
  if (threadIdx.x >= 3) return;
  const int a = threadIdx.x;
  float lo = INFINITY, hi = -INFINITY;
  for (uint32_t b = 0; b < nblk; ++b) {
    lo = fminf(lo, part[6 * b + a]);
    hi = fmaxf(hi, part[6 * b + 3 + a]);
  }
  const float e = __fsub_rn(hi, lo);
  params[a] = lo;
  params[3 + a] = e > 0.f ? __fdiv_rn(1024.0f, e) : 0.f;
}

__device__ __forceinline__ uint32_t quantise(float c, float lo, float scale) {
  const float q = __fmul_rn(__fsub_rn(c, lo), scale);
  if (!(q > 0.f)) return 0u;
  return min(__float2uint_rz(q), 1023u);
}

__global__ void k_morton(const float* __restrict__ cen, uint32_t n, const float* __restrict__ params,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const uint32_t qx = quantise(cen[3 * size_t(t)], params[0], params[3]);
  const uint32_t qy = quantise(cen[3 * size_t(t) + 1], params[1], params[4]);
  const uint32_t qz = quantise(cen[3 * size_t(t) + 2], params[2], params[5]);
  keys[t] = (expand_bits10(qx) << 2) | (expand_bits10(qy) << 1) | expand_bits10(qz);
  vals[t] = t;
}

// ---- stable LSD radix sort, 8 bits per pass ------------------------------------
__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                        uint32_t* __restrict__ hist, uint32_t nblk) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * kRsTile;
  const uint32_t end = min(n, base + kRsTile);
  for (uint32_t i = base + threadIdx.x; i < end; i += kRsThreads) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  __syncthreads();
  hist[size_t(threadIdx.x) * nblk + blockIdx.x] = h[threadIdx.x];
}

// Single-CTA exclusive scan of a u32 array in place.
__global__ void __launch_bounds__(1024) k_scan_exclusive(uint32_t* __restrict__ a, uint32_t total) {
  __shared__ uint32_t sums[1024];
  const uint32_t per = (total + 1023) / 1024;
  const uint32_t b = threadIdx.x * per, e = min(total, b + per);
  uint32_t s = 0;
  for (uint32_t i = b; i < e; ++i) s += a[i];
  sums[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const uint32_t v = threadIdx.x >= uint32_t(off) ? sums[threadIdx.x - off] : 0u;
    __syncthreads();
    sums[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = sums[threadIdx.x] - s;
  for (uint32_t i = b; i < e; ++i) {
    const uint32_t v = a[i];
    a[i] = run;
    run += v;
  }
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                           uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           uint32_t n, int shift, const uint32_t* __restrict__ hist,
                                                           uint32_t nblk) {
  constexpr int W = kRsThreads / 32;
  __shared__ uint32_t base[256];
  __shared__ uint32_t wcnt[W][256];
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  base[tid] = hist[size_t(tid) * nblk + blockIdx.x];
#pragma unroll
  for (int w = 0; w < W; ++w) wcnt[w][tid] = 0;
  __syncthreads();
  const uint32_t tile0 = blockIdx.x * kRsTile;
  for (uint32_t r = 0; r < kRsTile / kRsThreads; ++r) {
    const uint32_t i = tile0 + r * kRsThreads + tid;
    const bool valid = i < n;
    const uint32_t key = valid ? kin[i] : 0u;
    const uint32_t val = valid ? vin[i] : 0u;
    const uint32_t d = valid ? ((key >> shift) & 255u) : (256u + lane);
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & lanemask_lt());
    if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const uint32_t c = wcnt[w][tid];
      wcnt[w][tid] = run;
      run += c;
    }
    __syncthreads();
    if (valid) {
      const uint32_t dst = base[d] + wcnt[warp][d] + rank;
      kout[dst] = key;
      vout[dst] = val;
    }
    __syncthreads();
    base[tid] += run;
#pragma unroll
    for (int w = 0; w < W; ++w) wcnt[w][tid] = 0;
    __syncthreads();
  }
}

// `passes` stable 8-bit passes from bit 0; the sorted pairs end in (kin, vin)
// (the pointers are swapped in place).  Returns the number of kernels.
static int radix_passes(uint32_t*& kin, uint32_t*& vin, uint32_t*& kout, uint32_t*& vout, uint32_t n,
                        uint32_t* hist, int passes, cudaStream_t st) {
  const uint32_t nblk = (n + kRsTile - 1) / kRsTile;
  int L = 0;
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = 8 * pass;
    k_rs_hist<<<nblk, kRsThreads, 0, st>>>(kin, n, shift, hist, nblk); ++L;
    k_scan_exclusive<<<1, 1024, 0, st>>>(hist, nblk * 256); ++L;
    k_rs_scatter<<<nblk, kRsThreads, 0, st>>>(kin, vin, kout, vout, n, shift, hist, nblk); ++L;
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  return L;
}

// ---- probe ordering ------------------------------------------------------------------
// 24-bit Morton code of each probe position quantised inside the scene box;
// sorting by it groups spatially close probes into the same warp.
__global__ void k_probe_codes(const float* __restrict__ probes, uint32_t n, float lox, float loy, float loz,
                              float sx, float sy, float sz, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  auto q = [](float c, float lo, float s) -> uint32_t {
    const float v = (c - lo) * s;
    if (!(v > 0.f)) return 0u;
    return min(__float2uint_rz(v), 255u);
  };
  const uint32_t x = q(probes[3 * size_t(i)], lox, sx), y = q(probes[3 * size_t(i) + 1], loy, sy),
                 z = q(probes[3 * size_t(i) + 2], loz, sz);
  keys[i] = (expand_bits10(x) << 2) | (expand_bits10(y) << 1) | expand_bits10(z);
  vals[i] = i;
}

// Whole probe ordering in one CTA of 1024 threads for any n: codes, then three
// stable 8-bit LSD passes (histogram, scan, ranked scatter) through global
// ping-pong buffers, with the same warp ranking as k_rs_scatter.  Used for
// the batched bake's jobs above the counting sort's limit (one CTA per job).
__device__ __forceinline__ void probe_sort_cta(const float* __restrict__ probes, uint32_t n, float lox, float loy,
                                               float loz, float sx, float sy, float sz, uint32_t* ka, uint32_t* va,
                                               uint32_t* kb, uint32_t* vb, uint32_t* order) {
  constexpr int W = 32;
  __shared__ uint32_t base[256];
  __shared__ uint32_t wcnt[W][256];
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  auto q = [](float c, float lo, float s) -> uint32_t {
    const float v = (c - lo) * s;
    if (!(v > 0.f)) return 0u;
    return min(__float2uint_rz(v), 255u);
  };
  for (uint32_t i = tid; i < n; i += 1024) {
    const uint32_t x = q(probes[3 * size_t(i)], lox, sx), y = q(probes[3 * size_t(i) + 1], loy, sy),
                   z = q(probes[3 * size_t(i) + 2], loz, sz);
    ka[i] = (expand_bits10(x) << 2) | (expand_bits10(y) << 1) | expand_bits10(z);
    va[i] = i;
  }
  for (uint32_t j = tid; j < W * 256; j += 1024) wcnt[j / 256][j % 256] = 0;
  __syncthreads();
  for (int pass = 0; pass < 3; ++pass) {
    const int shift = 8 * pass;
    const uint32_t* kin = (pass & 1) ? kb : ka;
    const uint32_t* vin = (pass & 1) ? vb : va;
    uint32_t* kout = (pass & 1) ? ka : kb;
    uint32_t* vout = pass == 2 ? order : ((pass & 1) ? va : vb);
    if (tid < 256) base[tid] = 0;
    __syncthreads();
    for (uint32_t i = tid; i < n; i += 1024) atomicAdd(&base[(kin[i] >> shift) & 255u], 1u);
    __syncthreads();
    if (warp == 0) {  // exclusive scan of the 256 counts: 8 per lane
      uint32_t v[8], s = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) { v[j] = base[lane * 8 + j]; s += v[j]; }
      uint32_t incl = s;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= uint32_t(o)) incl += t;
      }
      uint32_t run = incl - s;
#pragma unroll
      for (int j = 0; j < 8; ++j) { base[lane * 8 + j] = run; run += v[j]; }
    }
    __syncthreads();
    for (uint32_t r0 = 0; r0 < n; r0 += 1024) {
      const uint32_t i = r0 + tid;
      const bool valid = i < n;
      const uint32_t key = valid ? kin[i] : 0u, val = valid ? vin[i] : 0u;
      const uint32_t d = valid ? ((key >> shift) & 255u) : (256u + lane);
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const uint32_t rank = __popc(peers & lanemask_lt());
      if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
      __syncthreads();
      uint32_t run = 0;
      if (tid < 256) {
        for (int w = 0; w < W; ++w) {
          const uint32_t c = wcnt[w][tid];
          wcnt[w][tid] = run;
          run += c;
        }
      }
      __syncthreads();
      if (valid) {
        const uint32_t dst = base[d] + wcnt[warp][d] + rank;
        kout[dst] = key;
        vout[dst] = val;
      }
      __syncthreads();
      if (tid < 256) {
        base[tid] += run;
        for (int w = 0; w < W; ++w) wcnt[w][tid] = 0;
      }
      __syncthreads();
    }
  }
}

// Probe order for n <= kCountMax probes in one CTA: a counting sort on the
// top 12 bits of the 24-bit Morton code (16^3 cells inside the bounds) with
// shared-memory histogram, scan and atomic cursors -- a handful of barriers
// instead of the radix sort's dozens.  The order inside a cell follows the
// atomics; the bake's results never depend on the probe order (each ray's
// walk and each probe's sums are independent of its packet), only its speed.
constexpr uint32_t kCountMax = 16384;
constexpr int kCountBins = 4096;

__device__ __forceinline__ void probe_sort_count(const float* __restrict__ probes, uint32_t n, float lox, float loy,
                                                 float loz, float sx, float sy, float sz,
                                                 uint32_t* __restrict__ order) {
  __shared__ uint32_t bin[kCountBins];
  __shared__ uint32_t wsum[32];
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  auto cell = [&](uint32_t i) -> uint32_t {
    auto q = [](float c, float lo, float s) -> uint32_t {
      const float v = (c - lo) * s;
      if (!(v > 0.f)) return 0u;
      return min(__float2uint_rz(v), 255u);
    };
    const uint32_t x = q(probes[3 * size_t(i)], lox, sx), y = q(probes[3 * size_t(i) + 1], loy, sy),
                   z = q(probes[3 * size_t(i) + 2], loz, sz);
    return ((expand_bits10(x) << 2) | (expand_bits10(y) << 1) | expand_bits10(z)) >> 12;
  };
  for (uint32_t b = tid; b < kCountBins; b += 1024) bin[b] = 0;
  __syncthreads();
  for (uint32_t i = tid; i < n; i += 1024) atomicAdd(&bin[cell(i)], 1u);
  __syncthreads();
  // exclusive scan: 4 bins per thread, warp shuffles, then the 32 warp totals
  uint32_t v[4], t = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) { v[k] = bin[4 * tid + k]; t += v[k]; }
  uint32_t incl = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= uint32_t(o)) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = wsum[lane];
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= uint32_t(o)) wi += y;
    }
    wsum[lane] = wi - w;
  }
  __syncthreads();
  uint32_t run = wsum[warp] + incl - t;
#pragma unroll
  for (int k = 0; k < 4; ++k) { bin[4 * tid + k] = run; run += v[k]; }
  __syncthreads();
  for (uint32_t i = tid; i < n; i += 1024) order[atomicAdd(&bin[cell(i)], 1u)] = i;
}

__global__ void __launch_bounds__(1024) k_probe_order_count(const float* __restrict__ probes, uint32_t n, float lox,
                                                             float loy, float loz, float sx, float sy, float sz,
                                                             uint32_t* __restrict__ order, uint32_t* zero_word) {
  if (threadIdx.x == 0 && zero_word) *zero_word = 0;  // the next kernel's work counter
  probe_sort_count(probes, n, lox, loy, loz, sx, sy, sz, order);
}

__global__ void __launch_bounds__(1024) k_probe_order_batch(const BakeJobDev* __restrict__ jobs) {
  const BakeJobDev& j = jobs[blockIdx.x];
  const uint32_t n = j.nprobes;
  float s[3];
  for (int i = 0; i < 3; ++i) {
    const float e = j.bounds[3 + i] - j.bounds[i];
    s[i] = e > 0.f ? 256.0f / e : 0.f;
  }
  if (n <= kCountMax) {
    probe_sort_count(j.probes, n, j.bounds[0], j.bounds[1], j.bounds[2], s[0], s[1], s[2], j.order);
    return;
  }
  uint32_t* sc = j.sort_scratch;  // 4 arrays of n
  probe_sort_cta(j.probes, n, j.bounds[0], j.bounds[1], j.bounds[2], s[0], s[1], s[2], sc, sc + n, sc + 2 * size_t(n),
                 sc + 3 * size_t(n), j.order);
}

void launch_probe_order_batch(const BakeJobDev* jobs, uint32_t njobs, cudaStream_t s) {
  if (njobs) k_probe_order_batch<<<njobs, 1024, 0, s>>>(jobs);
}

size_t probe_order_scratch_bytes(uint32_t n) {
  const uint32_t nblk = (n + kRsTile - 1) / kRsTile;
  const size_t a = (size_t(n) * 4 + 255) / 256 * 256;
  // multi-pass radix sort (above the counting sort's limit): 3 key/value buffers + histogram
  return 3 * a + size_t(nblk) * 256 * 4;
}

int launch_probe_order(const float* probes, uint32_t n, const float bounds[6], uint32_t* order, void* scratch,
                       uint32_t* zero_word, cudaStream_t st) {
  if (n == 0) {
    if (zero_word) cudaMemsetAsync(zero_word, 0, 4, st);
    return 0;
  }
  const size_t a = (size_t(n) * 4 + 255) / 256 * 256;
  char* base = static_cast<char*>(scratch);
  uint32_t* ka = reinterpret_cast<uint32_t*>(base);
  uint32_t* kb = reinterpret_cast<uint32_t*>(base + a);
  uint32_t* vb = reinterpret_cast<uint32_t*>(base + 2 * a);
  uint32_t* hist = reinterpret_cast<uint32_t*>(base + 3 * a);
  float s[3];
  for (int i = 0; i < 3; ++i) {
    const float e = bounds[3 + i] - bounds[i];
    s[i] = e > 0.f ? 256.0f / e : 0.f;
  }
  if (n <= kCountMax) {
    k_probe_order_count<<<1, 1024, 0, st>>>(probes, n, bounds[0], bounds[1], bounds[2], s[0], s[1], s[2], order,
                                            zero_word);
    return 1;
  }
  if (zero_word) cudaMemsetAsync(zero_word, 0, 4, st);
  k_probe_codes<<<(n + 255) / 256, 256, 0, st>>>(probes, n, bounds[0], bounds[1], bounds[2], s[0], s[1], s[2], ka,
                                                 order);
  uint32_t *kin = ka, *vin = order, *kout = kb, *vout = vb;
  // 24-bit keys: 3 passes; the odd pass count leaves the result in vb, copy it back
  int L = 1 + radix_passes(kin, vin, kout, vout, n, hist, 3, st);
  if (vin != order) cudaMemcpyAsync(order, vin, size_t(n) * 4, cudaMemcpyDeviceToDevice, st);
  return L;
}

// ---- Karras split search ---------------------------------------------------------
__device__ __forceinline__ int kdelta(const uint32_t* __restrict__ k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = k[i], b = k[j];
  if (a == b) return 32 + __clz(uint32_t(i) ^ uint32_t(j));
  return __clz(a ^ b);
}

__global__ void k_karras(const uint32_t* __restrict__ codes, int n, int32_t* __restrict__ child,
                         int32_t* __restrict__ parent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (kdelta(codes, n, i, i + 1) - kdelta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = kdelta(codes, n, i, i - d);
  int lmax = 2;
  while (kdelta(codes, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (kdelta(codes, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = kdelta(codes, n, i, j);
  int s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (kdelta(codes, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int g = i + s * d + min(d, 0);
  const int lo = min(i, j), hi = max(i, j);
  const int32_t left = (lo == g) ? ~int32_t(g) : int32_t(g);
  const int32_t right = (hi == g + 1) ? ~int32_t(g + 1) : int32_t(g + 1);
  child[2 * i] = left;
  child[2 * i + 1] = right;
  const int leaf0 = n - 1;
  parent[left >= 0 ? left : leaf0 + ~left] = i;
  parent[right >= 0 ? right : leaf0 + ~right] = i;
  if (i == 0) parent[0] = -1;
}

__global__ void k_leaf_boxes(const uint32_t* __restrict__ order, const float* __restrict__ tb, uint32_t n,
                             float* __restrict__ box) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t t = order[i];
#pragma unroll
  for (int a = 0; a < 6; ++a) box[6 * (size_t(n - 1) + i) + a] = tb[6 * size_t(t) + a];
}

__global__ void k_refit(const int32_t* __restrict__ parent, const int32_t* __restrict__ child, uint32_t n,
                        float* box, uint32_t* flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int leaf0 = int(n) - 1;
  int node = parent[leaf0 + int(i)];
  while (node >= 0) {
    __threadfence();
    if (atomicAdd(&flags[node], 1u) == 0u) return;  // first child to arrive stops here
    const int32_t c0 = child[2 * node], c1 = child[2 * node + 1];
    const float* b0 = box + 6 * size_t(c0 >= 0 ? c0 : leaf0 + ~c0);
    const float* b1 = box + 6 * size_t(c1 >= 0 ? c1 : leaf0 + ~c1);
    float* o = box + 6 * size_t(node);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      o[a] = fminf(__ldcg(b0 + a), __ldcg(b1 + a));
      o[3 + a] = fmaxf(__ldcg(b0 + 3 + a), __ldcg(b1 + 3 + a));
    }
    node = parent[node];
  }
}

// Traversal boxes are the exact boxes widened by (|x| + scene scale) * 2^-20
// per bound, so that the box tests are conservative: a ray lying in a box's
// face plane (a zero direction component) or grazing its boundary still
// enters it, and only the triangle test decides.  The exact boxes stay in
// `box` (exported and compared with the oracle).
__device__ __forceinline__ float widen_lo(float x, float scale) {
  return __fsub_rn(x, __fmul_rn(__fadd_rn(fabsf(x), scale), 0x1p-20f));
}
__device__ __forceinline__ float widen_hi(float x, float scale) {
  return __fadd_rn(x, __fmul_rn(__fadd_rn(fabsf(x), scale), 0x1p-20f));
}

__global__ void k_pack_nodes(const int32_t* __restrict__ child, const float* __restrict__ box, uint32_t n,
                             float4* __restrict__ nodes) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i + 1 >= n) return;
  const int leaf0 = int(n) - 1;
  const int32_t c0 = child[2 * i], c1 = child[2 * i + 1];
  const float* r = box;  // root (internal node 0)
  const float scale = fmaxf(fmaxf(fmaxf(fabsf(r[0]), fabsf(r[1])), fmaxf(fabsf(r[2]), fabsf(r[3]))),
                            fmaxf(fabsf(r[4]), fabsf(r[5])));
  const float* p0 = box + 6 * size_t(c0 >= 0 ? c0 : leaf0 + ~c0);
  const float* p1 = box + 6 * size_t(c1 >= 0 ? c1 : leaf0 + ~c1);
  float b0[6], b1[6];
  for (int a = 0; a < 3; ++a) {
    b0[a] = widen_lo(p0[a], scale); b0[3 + a] = widen_hi(p0[3 + a], scale);
    b1[a] = widen_lo(p1[a], scale); b1[3 + a] = widen_hi(p1[3 + a], scale);
  }
  pack_node(nodes + 4 * size_t(i), b0, b1, c0, c1);
}

__global__ void k_pack_tris(const uint32_t* __restrict__ order, const float* __restrict__ pos, uint32_t stride,
                            const uint32_t* __restrict__ idx, const float* __restrict__ albedo, uint32_t n,
                            float4* __restrict__ tris, float4* __restrict__ tri_albedo) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t t = order[i];
  const float* a = pos + size_t(idx[3 * t]) * stride;
  const float* b = pos + size_t(idx[3 * t + 1]) * stride;
  const float* c = pos + size_t(idx[3 * t + 2]) * stride;
  tris[3 * size_t(i) + 0] = make_float4(a[0], a[1], a[2], __int_as_float(int(t)));
  tris[3 * size_t(i) + 1] = make_float4(__fsub_rn(b[0], a[0]), __fsub_rn(b[1], a[1]), __fsub_rn(b[2], a[2]), 0.f);
  tris[3 * size_t(i) + 2] = make_float4(__fsub_rn(c[0], a[0]), __fsub_rn(c[1], a[1]), __fsub_rn(c[2], a[2]), 0.f);
  const float r = albedo ? albedo[3 * size_t(t)] : 1.f, g = albedo ? albedo[3 * size_t(t) + 1] : 1.f,
              bb = albedo ? albedo[3 * size_t(t) + 2] : 1.f;
  tri_albedo[t] = make_float4(r, g, bb, 0.f);
}

// ---- orchestration -------------------------------------------------------------------
struct LbvhScratch {
  float* tb; float* cen; float* part; float* params;
  uint32_t* ka; uint32_t* kb; uint32_t* va; uint32_t* vb;
  uint32_t* hist; int32_t* parent; uint32_t* flags;
};

static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

static size_t carve(uint32_t n, char* base, LbvhScratch* s) {
  const uint32_t nblk = (n + kRsTile - 1) / kRsTile;
  const uint32_t nred = 256;
  size_t off = 0;
  auto take = [&](size_t bytes) { char* p = base ? base + off : nullptr; off += align256(bytes); return p; };
  s->tb = reinterpret_cast<float*>(take(size_t(n) * 6 * 4));
  s->cen = reinterpret_cast<float*>(take(size_t(n) * 3 * 4));
  s->part = reinterpret_cast<float*>(take(size_t(nred) * 6 * 4));
  s->params = reinterpret_cast<float*>(take(6 * 4));
  s->ka = reinterpret_cast<uint32_t*>(take(size_t(n) * 4));
  s->kb = reinterpret_cast<uint32_t*>(take(size_t(n) * 4));
  s->va = reinterpret_cast<uint32_t*>(take(size_t(n) * 4));
  s->vb = reinterpret_cast<uint32_t*>(take(size_t(n) * 4));
  s->hist = reinterpret_cast<uint32_t*>(take(size_t(nblk) * 256 * 4));
  s->parent = reinterpret_cast<int32_t*>(take(size_t(2 * n) * 4));
  s->flags = reinterpret_cast<uint32_t*>(take(size_t(n) * 4));
  return off;
}

size_t lbvh_scratch_bytes(uint32_t ntris) {
  LbvhScratch s;
  return carve(ntris, nullptr, &s);
}

void launch_lbvh_build(const LbvhBuild& b, cudaStream_t st, int* launches) {
  const uint32_t n = b.ntris;
  if (n == 0) return;
  LbvhScratch s;
  carve(n, static_cast<char*>(b.scratch), &s);
  const uint32_t g = (n + 255) / 256;
  int L = 0;
  k_tri_bounds<<<g, 256, 0, st>>>(b.positions, b.stride_floats, b.indices, n, s.tb, s.cen); ++L;
  const uint32_t nred = min(256u, (n + kRedThreads - 1) / kRedThreads);
  k_cbounds_partial<<<nred, kRedThreads, 0, st>>>(s.cen, n, s.part); ++L;
  k_cbounds_final<<<1, 32, 0, st>>>(s.part, nred, s.params); ++L;
  k_morton<<<g, 256, 0, st>>>(s.cen, n, s.params, s.ka, s.va); ++L;
  uint32_t *kin = s.ka, *kout = s.kb, *vin = s.va, *vout = s.vb;
  L += radix_passes(kin, vin, kout, vout, n, s.hist, 4, st);
  cudaMemcpyAsync(b.codes, kin, size_t(n) * 4, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(b.order, vin, size_t(n) * 4, cudaMemcpyDeviceToDevice, st);
  k_leaf_boxes<<<g, 256, 0, st>>>(b.order, s.tb, n, b.box); ++L;
  if (n > 1) {
    const uint32_t gi = (n - 1 + 255) / 256;
    k_karras<<<gi, 256, 0, st>>>(b.codes, int(n), b.child, s.parent); ++L;
    cudaMemsetAsync(s.flags, 0, size_t(n) * 4, st);
    k_refit<<<g, 256, 0, st>>>(s.parent, b.child, n, b.box, s.flags); ++L;
    k_pack_nodes<<<gi, 256, 0, st>>>(b.child, b.box, n, b.nodes); ++L;
  }
  k_pack_tris<<<g, 256, 0, st>>>(b.order, b.positions, b.stride_floats, b.indices, b.albedo, n, b.tris,
                                 b.tri_albedo); ++L;
  if (launches) *launches += L;
}

}  // namespace vlbk
