// k_skybox.cu -- skybox SH projection (shaders/skybox_sh.comp:23-42,
// shaders/sh.comp:23-42 for the env-map form; Skybox_t::computeSH,
// src/skybox_manager.cpp:107-130).
//
// The reference lets every texel do an unsynchronised read-modify-write of
// the 48 output floats (skybox_sh.comp:39), so its result depends on
// scheduling.  Here each CTA owns a contiguous slab of texels, streams it
// through shared memory with 1-D bulk async copies (cp.async.bulk, completion
// on an mbarrier, 4 stages), evaluates the basis per texel in FP32, reduces
// with warp shuffles, writes one partial per slab, and a second kernel sums
// the slabs of each map in FP64 in a fixed order.  The result is identical
// run to run and independent of how many maps are batched together.
#include "vlb_device.cuh"
#include "vlb_internal.h"

namespace vlbk {

constexpr int kSkyThreads = 256;
constexpr int kSkyChunk = 1024;  // texels per pipeline stage, 4 per thread
constexpr int kSkyStages = 4;

// Exact solid angle of cube-face texel (x, y) of an n x n face, in FP64:
// corner sum of atan2(u v, sqrt(u^2 + v^2 + 1)), the antiderivative of the
// face area element (1 + u^2 + v^2)^(-3/2).
__global__ void k_cube_solid_angle(float* out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * n) return;
  const uint32_t x = i % n, y = i / n;
  const double s = 2.0 / double(n);
  const double u0 = -1.0 + s * x, u1 = u0 + s, v0 = -1.0 + s * y, v1 = v0 + s;
  auto A = [](double u, double v) { return atan2(u * v, sqrt(u * u + v * v + 1.0)); };
  out[i] = float(A(u0, v0) - A(u0, v1) - A(u1, v0) + A(u1, v1));
}

void launch_cube_solid_angle(float* out, uint32_t n, cudaStream_t s) {
  const uint32_t total = n * n;
  k_cube_solid_angle<<<(total + 255) / 256, 256, 0, s>>>(out, n);
}

struct SlabIter {
  uint32_t unit, chunk, seq;
};

template <int LMAX, int LAYOUT, int FMT, bool TMA>
__global__ void __launch_bounds__(kSkyThreads) k_skybox_sh(const SkyboxArgs a) {
  constexpr int K = sh_k<LMAX>();
  constexpr int V = 3 * K;
  constexpr int TB = FMT == 0 ? 12 : 4;  // bytes per texel
  extern __shared__ __align__(128) unsigned char stage_mem[];
  __shared__ __align__(8) uint64_t bars[kSkyStages];
  __shared__ float red[kSkyThreads / 32][V];

  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t units = a.count * a.slabs_per_map;
  const uint32_t T = a.texels_per_map;

  auto unit_range = [&](uint32_t u, uint32_t* t0, uint32_t* nchunks) {
    const uint32_t j = u % a.slabs_per_map;
    *t0 = j * a.slab_texels;
    const uint32_t t1 = min(T, *t0 + a.slab_texels);
    *nchunks = (t1 - *t0 + kSkyChunk - 1) / kSkyChunk;
  };
  auto chunk_texels = [&](uint32_t u, uint32_t c) -> uint32_t {
    uint32_t t0, nc;
    unit_range(u, &t0, &nc);
    const uint32_t t1 = min(T, t0 + a.slab_texels);
    const uint32_t b = t0 + c * kSkyChunk;
    return min(uint32_t(kSkyChunk), t1 - b);
  };
  auto advance = [&](SlabIter& it) {
    uint32_t t0, nc;
    unit_range(it.unit, &t0, &nc);
    ++it.seq;
    if (++it.chunk == nc) { it.chunk = 0; it.unit += gridDim.x; }
  };

  SlabIter prod{blockIdx.x, 0, 0};
  auto issue = [&](SlabIter& it) {
    const uint32_t st = it.seq % kSkyStages;
    uint32_t t0, nc;
    unit_range(it.unit, &t0, &nc);
    const uint32_t nt = chunk_texels(it.unit, it.chunk);
    const uint32_t m = it.unit / a.slabs_per_map;
    const size_t first = size_t(m) * T + t0 + size_t(it.chunk) * kSkyChunk;
    const unsigned char* src = static_cast<const unsigned char*>(a.texels) + first * TB;
    mbar_arrive_expect_tx(&bars[st], nt * TB);
    bulk_g2s(stage_mem + size_t(st) * kSkyChunk * TB, src, nt * TB, &bars[st]);
    advance(it);
  };

  if constexpr (TMA) {
    if (tid == 0) {
      for (int i = 0; i < kSkyStages; ++i) mbar_init(&bars[i], 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0)
      for (int i = 0; i < kSkyStages && prod.unit < units; ++i) issue(prod);
  }

  float acc[V];
#pragma unroll
  for (int v = 0; v < V; ++v) acc[v] = 0.f;

  const bool swap_rb = (a.flags & VLB_SKY_REF_BGRA_SWAP) != 0;
  const float inv255 = 1.0f / 255.0f;
  bool timed_out = false;

  SlabIter cons{blockIdx.x, 0, 0};
  while (cons.unit < units) {
    uint32_t t0, nc;
    unit_range(cons.unit, &t0, &nc);
    const uint32_t nt = chunk_texels(cons.unit, cons.chunk);
    const uint32_t m = cons.unit / a.slabs_per_map;
    const uint32_t tbase = t0 + cons.chunk * kSkyChunk;  // texel index within the map
    const uint32_t st = cons.seq % kSkyStages;
    bool ok = true;
    if constexpr (TMA) ok = mbar_wait_bounded(&bars[st], (cons.seq / kSkyStages) & 1u, a.err);
    const unsigned char* sbase = TMA ? stage_mem + size_t(st) * kSkyChunk * TB
                                     : static_cast<const unsigned char*>(a.texels) + (size_t(m) * T + tbase) * TB;
    if (ok) {
#pragma unroll
      for (int r = 0; r < kSkyChunk / kSkyThreads; ++r) {
        const uint32_t i = tid + r * kSkyThreads;
        if (i < nt) {
          float cr, cg, cb;
          if constexpr (FMT == 0) {
            const float* p = reinterpret_cast<const float*>(sbase) + 3 * i;
            cr = p[0]; cg = p[1]; cb = p[2];
          } else {
            const uchar4 q = reinterpret_cast<const uchar4*>(sbase)[i];
            cr = q.x * inv255; cg = q.y * inv255; cb = q.z * inv255;
          }
          if (swap_rb) { const float tmp = cr; cr = cb; cb = tmp; }
          const uint32_t t = tbase + i;
          float bx, by, bz, w;
          if constexpr (LAYOUT == VLB_SKY_CUBEMAP) {
            const uint32_t n = a.w, nn = n * n;
            const uint32_t face = t / nn, rem = t - face * nn, y = rem / n, x = rem - y * n;
            const float inv_n = 1.0f / float(n);
            const float u = fmaf(float(x), 2.0f * inv_n, inv_n - 1.0f);
            const float v = fmaf(float(y), 2.0f * inv_n, inv_n - 1.0f);
            const float rn = rsqrtf(fmaf(u, u, fmaf(v, v, 1.0f)));
            switch (face) {
              case 0: bx = rn; by = -v * rn; bz = -u * rn; break;
              case 1: bx = -rn; by = -v * rn; bz = u * rn; break;
              case 2: bx = u * rn; by = rn; bz = v * rn; break;
              case 3: bx = u * rn; by = -rn; bz = -v * rn; break;
              case 4: bx = u * rn; by = -v * rn; bz = rn; break;
              default: bx = -u * rn; by = -v * rn; bz = -rn; break;
            }
            w = __ldg(a.solid_angle + rem);
          } else {
            const uint32_t y = t / a.w, x = t - y * a.w;
            const float2 cs = __ldg(a.col_tab + x);
            const float4 rw = __ldg(a.row_tab + y);
            const float dx = rw.x * cs.x, dy = rw.x * cs.y, dz = rw.y;
            if constexpr (LAYOUT == VLB_SKY_PANORAMA) { bx = dx; by = dz; bz = dy; }  // skybox_sh.comp:39 dir.xzy
            else { bx = dx; by = dy; bz = dz; }
            w = rw.z;
          }
          float Y[K];
          sh_basis<LMAX>(bx, by, bz, Y);
          const float wr = w * cr, wg = w * cg, wb = w * cb;
#pragma unroll
          for (int k = 0; k < K; ++k) {
            acc[3 * k] = fmaf(Y[k], wr, acc[3 * k]);
            acc[3 * k + 1] = fmaf(Y[k], wg, acc[3 * k + 1]);
            acc[3 * k + 2] = fmaf(Y[k], wb, acc[3 * k + 2]);
          }
        }
      }
    }
    const bool last = cons.chunk + 1 == nc;
    if constexpr (TMA) {
      if (__syncthreads_or(!ok)) { timed_out = true; break; }
      if (tid == 0 && prod.unit < units) issue(prod);  // refill the stage just drained
    }
    if (last) {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const float s = warp_sum(acc[v]);
        if (lane == 0) red[warp][v] = s;
        acc[v] = 0.f;
      }
      __syncthreads();
      if (tid < V) {
        float s = 0.f;
#pragma unroll
        for (int w = 0; w < kSkyThreads / 32; ++w) s += red[w][tid];
        a.partial[size_t(cons.unit) * V + tid] = s;
      }
      __syncthreads();
    }
    advance(cons);
  }
  if constexpr (TMA) {
    // After a timeout, let copies already issued land before the CTA exits.
    if (timed_out && tid == 0) {
      for (uint32_t q = cons.seq; q < prod.seq; ++q)
        mbar_wait_bounded(&bars[q % kSkyStages], (q / kSkyStages) & 1u, a.err, 1u << 16);
    }
  }
}

template <int LMAX, int LAYOUT, int FMT>
static void launch3(const SkyboxArgs& a, bool tma, int grid, cudaStream_t s) {
  const int TB = FMT == 0 ? 12 : 4;
  const size_t smem = tma ? size_t(kSkyStages) * kSkyChunk * TB : 0;
  if (tma) {
    auto k = k_skybox_sh<LMAX, LAYOUT, FMT, true>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    k<<<grid, kSkyThreads, smem, s>>>(a);
  } else {
    k_skybox_sh<LMAX, LAYOUT, FMT, false><<<grid, kSkyThreads, 0, s>>>(a);
  }
}

template <int LMAX, int LAYOUT>
static void launch2(const SkyboxArgs& a, bool tma, int grid, cudaStream_t s) {
  if (a.fmt == VLB_TEXEL_RGB32F) launch3<LMAX, LAYOUT, 0>(a, tma, grid, s);
  else launch3<LMAX, LAYOUT, 1>(a, tma, grid, s);
}

template <int LMAX>
static void launch1(const SkyboxArgs& a, bool tma, int grid, cudaStream_t s) {
  switch (a.layout) {
    case VLB_SKY_CUBEMAP: launch2<LMAX, VLB_SKY_CUBEMAP>(a, tma, grid, s); break;
    case VLB_SKY_PANORAMA: launch2<LMAX, VLB_SKY_PANORAMA>(a, tma, grid, s); break;
    default: launch2<LMAX, VLB_SKY_ENVMAP>(a, tma, grid, s); break;
  }
}

int launch_skybox_sh(const SkyboxArgs& a, bool tma, int num_sms, cudaStream_t s) {
  const uint32_t units = a.count * a.slabs_per_map;
  const uint64_t cap = uint64_t(num_sms) * 4;
  const int grid = int(units < cap ? units : cap);
  if (a.lmax == 2) launch1<2>(a, tma, grid, s);
  else launch1<3>(a, tma, grid, s);
  return grid;
}

__global__ void k_sh_finalize(const float* partial, uint32_t nmaps, uint32_t slabs, uint32_t nvals, float* out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nmaps * nvals) return;
  const uint32_t m = i / nvals, v = i - m * nvals;
  const float* p = partial + size_t(m) * slabs * nvals + v;
  double s = 0.0;
  for (uint32_t j = 0; j < slabs; ++j) s += double(p[size_t(j) * nvals]);
  out[i] = float(s);
}

void launch_sh_finalize(const float* partial, uint32_t nmaps, uint32_t slabs, uint32_t nvals, float* out,
                        cudaStream_t s) {
  const uint32_t total = nmaps * nvals;
  k_sh_finalize<<<(total + 255) / 256, 256, 0, s>>>(partial, nmaps, slabs, nvals, out);
}

}  // namespace vlbk
