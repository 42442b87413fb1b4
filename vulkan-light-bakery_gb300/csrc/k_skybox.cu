// k_skybox.cu -- skybox SH projection (shaders/skybox_sh.comp:23-42,
// shaders/sh.comp:23-42 for the env-map form; Skybox_t::computeSH,
// src/skybox_manager.cpp:107-130).
//
// The reference lets every texel do an unsynchronised read-modify-write of
// the 48 output floats (skybox_sh.comp:39), so its result depends on
// scheduling.  Here a work unit is a fixed slab of texels of a group of maps,
// and a CTA streams the group's texels through a shared-memory ring filled by
// 1-D bulk async copies (cp.async.bulk, completion on an mbarrier; one copy
// per map per stage) from a producer warp.  Cubemaps with faces up to 1024
// (k_skybox_cube_group) share one weighted-basis row, read from a texel-pair
// table, among 8-16 maps; panoramas, env maps and larger faces (k_skybox_sh)
// compute each texel's direction, solid angle and basis once and apply it to
// G = 1-4 maps with packed FP32x2 FMAs.  Each map's sums are reduced with warp
// shuffles into partials per (map, slab), and a second kernel adds a map's
// partials in FP64 in a fixed order.  The slab size does not depend on the
// batch, so a map's result is bit-identical alone or in any batch.
#include "vlb_device.cuh"
#include "vlb_internal.h"

namespace vlbk {

constexpr int kSkyConsumers = 32 * kSkyPartialsPerSlab;  // consumer threads (8 warps)
constexpr int kSkyThreads = kSkyConsumers + 32;           // + one producer warp
constexpr int kSkyChunk = 512;  // texels per map per pipeline stage, 2 per consumer thread
constexpr int kSkyStages = 3;
constexpr uint32_t kSkySlab = 8192;  // texels per work unit, independent of the batch
// k_skybox_cube_group (cubemap batches with the pair table)
constexpr int kGroupChunk = 256;          // texels per map per stage
constexpr int kGroupPairs = kGroupChunk / 2;
constexpr uint32_t kGroupSlab = 4096;     // texels per work unit

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

// Weighted basis of cubemap texel t (faces +X,-X,+Y,-Y,+Z,-Z) in FP64: the
// exact solid angle times the basis at the texel centre, constants of
// shaders/sh_common.h:26-116.  b[0..15] (the first (lmax+1)^2 are used).
__device__ void cube_texel_basis64(uint32_t t, uint32_t n, double* b) {
  const uint32_t nn = n * n, face = t / nn, rem = t - face * nn, y = rem / n, x = rem - y * n;
  const double s = 2.0 / double(n);
  const double u0 = -1.0 + s * x, u1 = u0 + s, v0 = -1.0 + s * y, v1 = v0 + s;
  auto A = [](double u, double v) { return atan2(u * v, sqrt(u * u + v * v + 1.0)); };
  const double w = A(u0, v0) - A(u0, v1) - A(u1, v0) + A(u1, v1);
  const double u = u0 + 0.5 * s, v = v0 + 0.5 * s;
  double d[3];
  switch (face) {
    case 0: d[0] = 1.0; d[1] = -v; d[2] = -u; break;
    case 1: d[0] = -1.0; d[1] = -v; d[2] = u; break;
    case 2: d[0] = u; d[1] = 1.0; d[2] = v; break;
    case 3: d[0] = u; d[1] = -1.0; d[2] = -v; break;
    case 4: d[0] = u; d[1] = -v; d[2] = 1.0; break;
    default: d[0] = -u; d[1] = -v; d[2] = -1.0; break;
  }
  const double r = 1.0 / sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const double X = d[0] * r, Yy = d[1] * r, Z = d[2] * r;
  const double c[16] = {0.282095, -0.488603 * Yy, 0.488603 * Z, -0.488603 * X, 1.092548 * X * Yy,
                        -1.092548 * Yy * Z, 0.315392 * (-X * X - Yy * Yy + 2.0 * Z * Z), -1.092548 * X * Z,
                        0.546274 * (X * X - Yy * Yy), -0.590044 * Yy * (3.0 * X * X - Yy * Yy), 2.890611 * X * Yy * Z,
                        -0.457046 * Yy * (4.0 * Z * Z - X * X - Yy * Yy),
                        0.373176 * Z * (2.0 * Z * Z - 3.0 * X * X - 3.0 * Yy * Yy),
                        -0.457046 * X * (4.0 * Z * Z - X * X - Yy * Yy), 1.445306 * Z * (X * X - Yy * Yy),
                        -0.590044 * X * (X * X - 3.0 * Yy * Yy)};
  for (int k = 0; k < 16; ++k) b[k] = w * c[k];
}

void skybox_plan(SkyboxArgs& a, uint32_t max_slabs) {
  uint32_t slab = a.pair_table ? kGroupSlab : kSkySlab;
  if (max_slabs && (a.texels_per_map + slab - 1) / slab > max_slabs)
    slab = ((a.texels_per_map + max_slabs - 1) / max_slabs + kSkyChunk - 1) / kSkyChunk * kSkyChunk;
  a.slab_texels = slab;
  a.slabs_per_map = (a.texels_per_map + slab - 1) / slab;
  // two maps per unit fill one packed FP32x2 pair and keep ~120 registers,
  // two CTAs per SM (four maps measured slower: ~190 registers, one CTA)
  a.group = a.count == 1 ? 1 : 2;
}

// q = num / d for num < 2^31 (float estimate, then exact integer correction)
__device__ __forceinline__ uint32_t udiv(uint32_t num, uint32_t d, float inv_d) {
  uint32_t q = __float2uint_rz(__fmul_rn(float(num) + 0.5f, inv_d));
  while (q * d > num) --q;
  while (num - q * d >= d) ++q;
  return q;
}

__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;"
      : "=l"(d)
      : "l"(*reinterpret_cast<uint64_t*>(&a)), "l"(*reinterpret_cast<uint64_t*>(&b)),
        "l"(*reinterpret_cast<uint64_t*>(&c)));
  return *reinterpret_cast<float2*>(&d);
}

template <int FMT>
__device__ __forceinline__ void texel_rgb(const unsigned char* p, uint32_t i, bool swap, float* c) {
  if constexpr (FMT == 0) {
    const float* f = reinterpret_cast<const float*>(p) + 3 * i;
    c[0] = f[0]; c[1] = f[1]; c[2] = f[2];
  } else {
    const uchar4 q = reinterpret_cast<const uchar4*>(p)[i];
    const float s = 1.0f / 255.0f;
    c[0] = q.x * s; c[1] = q.y * s; c[2] = q.z * s;
  }
  if (swap) { const float t = c[0]; c[0] = c[2]; c[2] = t; }
}

// Warp-specialised: warps 0..7 consume, warp 8 (TMA path) produces.  The
// producer refills a stage as soon as all 8 consumer warps have arrived on
// its `empty` barrier; consumers never wait for each other.  Each consumer
// warp reduces its own sums with shuffles and writes one partial per (map,
// slab, warp), so no CTA-wide barrier follows the set-up -- a consumer whose
// bounded wait gives up simply stops, and nobody is left waiting for it.
template <int LMAX, int LAYOUT, int FMT, int G, bool TMA>
__global__ void __launch_bounds__(kSkyThreads) k_skybox_sh(const SkyboxArgs a) {
  constexpr int K = sh_k<LMAX>();
  constexpr int V = 3 * K;
  constexpr int GP = (G + 1) / 2;  // map pairs
  constexpr int TB = FMT == 0 ? 12 : 4;
  constexpr uint32_t kMapChunkBytes = kSkyChunk * TB;
  constexpr uint32_t kStageBytes = G * kMapChunkBytes;  // G map chunks
  constexpr uint32_t kConsumerWarps = kSkyConsumers / 32;
  extern __shared__ __align__(128) unsigned char stage_mem[];
  __shared__ __align__(8) uint64_t full[kSkyStages], empty[kSkyStages];
  __shared__ volatile int abort_flag;

  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t T = a.texels_per_map, spm = a.slabs_per_map;
  const uint32_t groups = (a.count + G - 1) / G;
  const uint32_t units = groups * spm;
  const unsigned char* tex = static_cast<const unsigned char*>(a.texels);

  // (unit, chunk) iteration shared by the producer and the consumers
  struct It { uint32_t unit, chunk, seq; };
  auto nchunks = [&](uint32_t u) {
    const uint32_t t0 = (u % spm) * a.slab_texels, t1 = min(T, t0 + a.slab_texels);
    return (t1 - t0 + kSkyChunk - 1) / kSkyChunk;
  };
  auto advance = [&](It& it) {
    ++it.seq;
    if (++it.chunk == nchunks(it.unit)) { it.chunk = 0; it.unit += gridDim.x; }
  };
  auto chunk_span = [&](const It& it, uint32_t* tb, uint32_t* nt, uint32_t* m0, uint32_t* gv) {
    const uint32_t t0 = (it.unit % spm) * a.slab_texels, t1 = min(T, t0 + a.slab_texels);
    *tb = t0 + it.chunk * kSkyChunk;
    *nt = min(uint32_t(kSkyChunk), t1 - *tb);
    *m0 = (it.unit / spm) * G;
    *gv = min(uint32_t(G), a.count - *m0);
  };

  if (tid == 0) {
    for (int i = 0; i < kSkyStages; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], kConsumerWarps); }
    abort_flag = 0;
    fence_mbar_init();
  }
  __syncthreads();

  const uint32_t polls = a.wait_polls ? a.wait_polls : kWaitPolls;
  if (warp == kConsumerWarps) {  // producer warp
    if (TMA && lane == 0 && !a.hold_producer) {  // hold (a test hook): nothing is issued, consumers give up
      It it{blockIdx.x, 0, 0};
      while (it.unit < units && !abort_flag) {
        const uint32_t st = it.seq % kSkyStages;
        if (!mbar_wait_bounded(&empty[st], ((it.seq / kSkyStages) & 1u) ^ 1u, a.err, polls)) {
          abort_flag = 1;
          break;
        }
        uint32_t tb, nt, m0, gv;
        chunk_span(it, &tb, &nt, &m0, &gv);
        unsigned char* sbase = stage_mem + size_t(st) * kStageBytes;
        mbar_arrive_expect_tx(&full[st], gv * nt * TB);
        for (uint32_t g = 0; g < gv; ++g)
          bulk_g2s(sbase + g * kMapChunkBytes, tex + (size_t(m0 + g) * T + tb) * TB, nt * TB, &full[st]);
        advance(it);
      }
      // every copy issued lands before the CTA may exit
      const uint32_t first = it.seq > uint32_t(kSkyStages) ? it.seq - kSkyStages : 0;
      for (uint32_t q = first; q < it.seq; ++q)
        mbar_wait_bounded(&full[q % kSkyStages], (q / kSkyStages) & 1u, a.err, 1u << 16);
    }
    return;
  }

  float2 acc[GP][V];
#pragma unroll
  for (int p = 0; p < GP; ++p)
#pragma unroll
    for (int v = 0; v < V; ++v) acc[p][v] = make_float2(0.f, 0.f);

  const bool swap_rb = (a.flags & VLB_SKY_REF_BGRA_SWAP) != 0;
  const float inv_w = 1.0f / float(a.w);
  const uint32_t nn = a.w * a.w;
  const float inv_nn = 1.0f / float(nn);

  It cons{blockIdx.x, 0, 0};
  while (cons.unit < units) {
    uint32_t tb, nt, m0, gv;
    chunk_span(cons, &tb, &nt, &m0, &gv);
    const uint32_t st = cons.seq % kSkyStages;
    if constexpr (TMA) {
      if (!mbar_wait_bounded(&full[st], (cons.seq / kSkyStages) & 1u, a.err, polls)) abort_flag = 1;
    }
    if (abort_flag) break;
    const unsigned char* sbase = stage_mem + size_t(st) * kStageBytes;
    // per-chunk pointers: the group's texel chunks
    const unsigned char* mp[G];
#pragma unroll
    for (int g = 0; g < G; ++g)
      mp[g] = TMA ? sbase + g * kMapChunkBytes : tex + (size_t(m0 + min(uint32_t(g), gv - 1)) * T + tb) * TB;
    // chunk origin: one division per chunk, the texels then step from it
    uint32_t face0 = 0, rem0 = 0, y0 = 0, x0 = 0;
    if constexpr (LAYOUT == VLB_SKY_CUBEMAP) {
      face0 = udiv(tb, nn, inv_nn);
      rem0 = tb - face0 * nn;
    } else {
      y0 = udiv(tb, a.w, inv_w);
      x0 = tb - y0 * a.w;
    }
#pragma unroll 1
    for (uint32_t i = tid; i < nt; i += kSkyConsumers) {
      float Y[K];
      {
        float bx, by, bz, w;
        if constexpr (LAYOUT == VLB_SKY_CUBEMAP) {
          const uint32_t n = a.w;
          uint32_t rem = rem0 + i, face = face0;
          while (rem >= nn) { rem -= nn; ++face; }
          const uint32_t y = udiv(rem, n, inv_w), x = rem - y * n;
          const float u = fmaf(float(x), 2.0f * inv_w, inv_w - 1.0f);
          const float v = fmaf(float(y), 2.0f * inv_w, inv_w - 1.0f);
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
          const uint32_t xi = x0 + i;
          const uint32_t dy = udiv(xi, a.w, inv_w);
          const uint32_t x = xi - dy * a.w, y = y0 + dy;
          const float2 cs = __ldg(a.col_tab + x);
          const float4 rw = __ldg(a.row_tab + y);
          const float dx = rw.x * cs.x, dyy = rw.x * cs.y, dz = rw.y;
          if constexpr (LAYOUT == VLB_SKY_PANORAMA) { bx = dx; by = dz; bz = dyy; }  // skybox_sh.comp:39 dir.xzy
          else { bx = dx; by = dyy; bz = dz; }
          w = rw.z;
        }
        sh_basis<LMAX>(bx, by, bz, Y);
#pragma unroll
        for (int k = 0; k < K; ++k) Y[k] *= w;
      }
#pragma unroll
      for (int p = 0; p < GP; ++p) {
        float ca[3], cb[3] = {0.f, 0.f, 0.f};
        texel_rgb<FMT>(mp[2 * p], i, false, ca);
        if (2 * p + 1 < G) texel_rgb<FMT>(mp[2 * p + 1], i, false, cb);  // stale or repeated if gv < G: never written
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const float2 yk = make_float2(Y[k], Y[k]);
#pragma unroll
          for (int c = 0; c < 3; ++c) acc[p][3 * k + c] = ffma2(yk, make_float2(ca[c], cb[c]), acc[p][3 * k + c]);
        }
      }
    }
    if constexpr (TMA) {
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[st]);  // this warp is done with the stage
    }
    if (cons.chunk + 1 == nchunks(cons.unit)) {
      // the warp's partial for each map of the group: partial[map][slab][warp][v]
      const uint32_t slab = cons.unit % spm;
#pragma unroll
      for (int p = 0; p < GP; ++p)
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const float s0 = warp_sum(acc[p][v].x), s1 = warp_sum(acc[p][v].y);
          acc[p][v] = make_float2(0.f, 0.f);
          if (lane == 0) {
            const int k = v / 3, c = v - 3 * k;
            const int vo = 3 * k + (swap_rb ? 2 - c : c);  // R/B swap applied to the linear result
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const uint32_t g = 2 * p + h;
              if (g < gv && (h == 0 || 2 * p + 1 < G))
                a.partial[((size_t(m0 + g) * spm + slab) * kConsumerWarps + warp) * V + vo] = h ? s1 : s0;
            }
          }
        }
    }
    advance(cons);
  }
}

// Cubemap batches, 8 * MPW maps per work unit: consumer warp w owns maps
// MPW*w .. MPW*w + MPW - 1 of the group, and every warp reads the same
// per-texel weighted basis, so one basis row serves 8 * MPW maps (the
// basis stream is 9-16 floats a texel against 12 bytes a texel of every
// map).  The basis comes from a table in FP64 rounded once
// (cube_texel_basis64), laid out per 256-texel chunk for texel pairs: lane l
// of a warp takes texels 64b + l and 64b + 32 + l (b = 0..3) -- stride-3
// words across the lanes, so the texel reads are free of bank conflicts --
// and entry [chunk][k][32b + l] holds the pair's two weighted basis values
// as one float2, so each packed FP32x2 FMA adds both texels' products.  The
// producer warp streams, per stage, the table chunk and the group's texel
// chunks (1-D bulk copies into an NST-stage ring).  One partial per (map,
// slab), added in FP64 by k_sh_finalize: a map's result does not depend on
// the batch or on the map's place in it.

// The pair table: [chunk][k][p] float2 for chunks of kGroupChunk texels;
// texels past the map's end have weight 0.
__global__ void k_cube_pair_table(float2* out, uint32_t n, uint32_t lmax) {
  const uint32_t K = (lmax + 1) * (lmax + 1);
  const uint32_t T = 6 * n * n, chunks = (T + kGroupChunk - 1) / kGroupChunk;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= chunks * kGroupPairs) return;
  const uint32_t c = i / kGroupPairs, pr = i - c * kGroupPairs;
  const uint32_t t0 = c * kGroupChunk + 64 * (pr / 32) + pr % 32, t1 = t0 + 32;
  double b0[16] = {}, b1[16] = {};
  if (t0 < T) cube_texel_basis64(t0, n, b0);
  if (t1 < T) cube_texel_basis64(t1, n, b1);
  for (uint32_t k = 0; k < K; ++k)
    out[(size_t(c) * K + k) * kGroupPairs + pr] = make_float2(float(b0[k]), float(b1[k]));
}

size_t cube_pair_table_bytes(uint32_t n, uint32_t lmax) {
  const size_t chunks = (size_t(6) * n * n + kGroupChunk - 1) / kGroupChunk;
  return chunks * size_t(lmax + 1) * (lmax + 1) * kGroupPairs * sizeof(float2);
}

void launch_cube_pair_table(float2* out, uint32_t n, uint32_t lmax, cudaStream_t s) {
  const uint32_t total = uint32_t((size_t(6) * n * n + kGroupChunk - 1) / kGroupChunk) * kGroupPairs;
  k_cube_pair_table<<<(total + 255) / 256, 256, 0, s>>>(out, n, lmax);
}

template <int LMAX, int FMT, int MPW, int NST>
__global__ void __launch_bounds__(kSkyThreads) k_skybox_cube_group(const SkyboxArgs a) {
  constexpr int K = sh_k<LMAX>();
  constexpr int V = 3 * K;
  constexpr int TB = FMT == 0 ? 12 : 4;
  constexpr uint32_t kConsumerWarps = kSkyConsumers / 32;
  constexpr int G = int(kConsumerWarps) * MPW;
  constexpr uint32_t kMapChunkBytes = kGroupChunk * TB;
  constexpr uint32_t kTabBytes = K * kGroupPairs * 8;
  constexpr uint32_t kStageBytes = kTabBytes + G * kMapChunkBytes;  // the table chunk, then the maps
  constexpr int kStages = NST;
  extern __shared__ __align__(128) unsigned char stage_mem[];
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages];
  __shared__ volatile int abort_flag;

  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t T = a.texels_per_map, spm = a.slabs_per_map;
  const uint32_t groups = (a.count + G - 1) / G;
  const uint32_t units = groups * spm;
  const unsigned char* tex = static_cast<const unsigned char*>(a.texels);
  const unsigned char* tab = reinterpret_cast<const unsigned char*>(a.pair_table);
  const uint32_t polls = a.wait_polls ? a.wait_polls : kWaitPolls;

  struct It { uint32_t unit, chunk, seq; };
  auto nchunks = [&](uint32_t u) {
    const uint32_t t0 = (u % spm) * a.slab_texels, t1 = min(T, t0 + a.slab_texels);
    return (t1 - t0 + kGroupChunk - 1) / kGroupChunk;
  };
  auto advance = [&](It& it) {
    ++it.seq;
    if (++it.chunk == nchunks(it.unit)) { it.chunk = 0; it.unit += gridDim.x; }
  };
  auto chunk_span = [&](const It& it, uint32_t* tb, uint32_t* nt, uint32_t* m0, uint32_t* gv) {
    const uint32_t t0 = (it.unit % spm) * a.slab_texels, t1 = min(T, t0 + a.slab_texels);
    *tb = t0 + it.chunk * kGroupChunk;
    *nt = min(uint32_t(kGroupChunk), t1 - *tb);
    *m0 = (it.unit / spm) * G;
    *gv = min(uint32_t(G), a.count - *m0);
  };

  if (tid == 0) {
    for (int i = 0; i < kStages; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], kConsumerWarps); }
    abort_flag = 0;
    fence_mbar_init();
  }
  __syncthreads();

  if (warp == kConsumerWarps) {  // producer warp
    if (lane == 0 && !a.hold_producer) {  // hold (a test hook): nothing is issued, consumers give up
      It it{blockIdx.x, 0, 0};
      while (it.unit < units && !abort_flag) {
        const uint32_t st = it.seq % kStages;
        if (!mbar_wait_bounded(&empty[st], ((it.seq / kStages) & 1u) ^ 1u, a.err, polls)) {
          abort_flag = 1;
          break;
        }
        uint32_t tb, nt, m0, gv;
        chunk_span(it, &tb, &nt, &m0, &gv);
        unsigned char* sbase = stage_mem + size_t(st) * kStageBytes;
        mbar_arrive_expect_tx(&full[st], kTabBytes + gv * nt * TB);
        bulk_g2s(sbase, tab + size_t(tb / kGroupChunk) * kTabBytes, kTabBytes, &full[st]);
        for (uint32_t g = 0; g < gv; ++g)
          bulk_g2s(sbase + kTabBytes + g * kMapChunkBytes, tex + (size_t(m0 + g) * T + tb) * TB, nt * TB,
                   &full[st]);
        advance(it);
      }
      // every copy issued lands before the CTA may exit
      const uint32_t first = it.seq > uint32_t(kStages) ? it.seq - kStages : 0;
      for (uint32_t q = first; q < it.seq; ++q)
        mbar_wait_bounded(&full[q % kStages], (q / kStages) & 1u, a.err, 1u << 16);
    }
    return;
  }

  float2 acc[MPW][V];
#pragma unroll
  for (int m = 0; m < MPW; ++m)
#pragma unroll
    for (int v = 0; v < V; ++v) acc[m][v] = make_float2(0.f, 0.f);
  const bool swap_rb = (a.flags & VLB_SKY_REF_BGRA_SWAP) != 0;

  It cons{blockIdx.x, 0, 0};
  while (cons.unit < units) {
    uint32_t tb, nt, m0, gv;
    chunk_span(cons, &tb, &nt, &m0, &gv);
    const uint32_t st = cons.seq % kStages;
    if (!mbar_wait_bounded(&full[st], (cons.seq / kStages) & 1u, a.err, polls)) abort_flag = 1;
    if (abort_flag) break;
    const unsigned char* sbase = stage_mem + size_t(st) * kStageBytes;
    const float2* ytab = reinterpret_cast<const float2*>(sbase);
    if (MPW * warp < gv) {  // this warp owns at least one map of the group
#pragma unroll
      for (int b = 0; b < kGroupPairs / 32; ++b) {
        const uint32_t i0 = 64 * b + lane, i1 = i0 + 32;
        if (nt < uint32_t(kGroupChunk) && i0 >= nt) break;  // a map's last, partial chunk
        float2 yk[K];
#pragma unroll
        for (int k = 0; k < K; ++k) yk[k] = ytab[k * kGroupPairs + 32 * b + lane];
#pragma unroll
        for (int m = 0; m < MPW; ++m) {
          // stale for maps past gv and texels past nt: their products are never written
          const unsigned char* mp = sbase + kTabBytes + (MPW * warp + m) * kMapChunkBytes;
          float c0[3], c1[3];
          texel_rgb<FMT>(mp, i0, false, c0);
          texel_rgb<FMT>(mp, i1, false, c1);
          if (nt < uint32_t(kGroupChunk) && i1 >= nt) { c1[0] = c1[1] = c1[2] = 0.f; }
#pragma unroll
          for (int k = 0; k < K; ++k)
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[m][3 * k + c] = ffma2(yk[k], make_float2(c0[c], c1[c]), acc[m][3 * k + c]);
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);  // this warp is done with the stage
    if (cons.chunk + 1 == nchunks(cons.unit)) {
      const uint32_t slab = cons.unit % spm;
#pragma unroll
      for (int m = 0; m < MPW; ++m) {
        const uint32_t g = MPW * warp + m;
#pragma unroll
        for (int vv = 0; vv < V; ++vv) {
          const float s = warp_sum(acc[m][vv].x + acc[m][vv].y);
          acc[m][vv] = make_float2(0.f, 0.f);
          if (lane == 0 && g < gv) {
            const int k = vv / 3, c = vv - 3 * k;
            const int vo = 3 * k + (swap_rb ? 2 - c : c);  // R/B swap applied to the linear result
            a.partial[(size_t(m0 + g) * spm + slab) * V + vo] = s;
          }
        }
      }
    }
    advance(cons);
  }
}

template <int LMAX, int FMT, int MPW, int NST>
static void launch_group(const SkyboxArgs& a, int num_sms, cudaStream_t s) {
  constexpr int K = sh_k<LMAX>();
  constexpr int G = kSkyPartialsPerSlab * MPW;
  const int TB = FMT == 0 ? 12 : 4;
  const size_t smem = size_t(NST) * (size_t(K) * kGroupPairs * 8 + size_t(G) * kGroupChunk * TB);
  const uint32_t groups = (a.count + G - 1) / G;
  const uint64_t units = uint64_t(groups) * a.slabs_per_map;
  auto k = k_skybox_cube_group<LMAX, FMT, MPW, NST>;
  static std::atomic<uint64_t> opted{0};
  smem_opt_in(k, int(smem), opted);
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kSkyThreads, smem);
  if (per_sm < 1) per_sm = 1;
  const uint64_t cap = uint64_t(num_sms) * per_sm;
  k<<<int(units < cap ? units : cap), kSkyThreads, smem, s>>>(a);
}

template <int LMAX, int LAYOUT, int FMT, int G>
static void launch4(const SkyboxArgs& a, bool tma, int num_sms, cudaStream_t s) {
  const int TB = FMT == 0 ? 12 : 4;
  const size_t smem = tma ? size_t(kSkyStages) * (G * kSkyChunk * TB) : 0;
  const uint32_t groups = (a.count + G - 1) / G;
  const uint64_t units = uint64_t(groups) * a.slabs_per_map;
  auto k = tma ? k_skybox_sh<LMAX, LAYOUT, FMT, G, true> : k_skybox_sh<LMAX, LAYOUT, FMT, G, false>;
  if (smem) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kSkyThreads, smem);
  if (per_sm < 1) per_sm = 1;
  const uint64_t cap = uint64_t(num_sms) * per_sm;
  const int grid = int(units < cap ? units : cap);
  k<<<grid, kSkyThreads, smem, s>>>(a);
}

template <int LMAX, int LAYOUT, int FMT>
static void launch3(const SkyboxArgs& a, bool tma, int num_sms, cudaStream_t s) {
  if (a.group == 1) launch4<LMAX, LAYOUT, FMT, 1>(a, tma, num_sms, s);
  else if (LMAX == 2 && a.group == 4) launch4<LMAX, LAYOUT, FMT, 4>(a, tma, num_sms, s);
  else launch4<LMAX, LAYOUT, FMT, 2>(a, tma, num_sms, s);
}

template <int LMAX, int LAYOUT>
static void launch2(const SkyboxArgs& a, bool tma, int num_sms, cudaStream_t s) {
  if (a.fmt == VLB_TEXEL_RGB32F) launch3<LMAX, LAYOUT, 0>(a, tma, num_sms, s);
  else launch3<LMAX, LAYOUT, 1>(a, tma, num_sms, s);
}

template <int LMAX>
static void launch1(const SkyboxArgs& a, bool tma, int num_sms, cudaStream_t s) {
  switch (a.layout) {
    case VLB_SKY_CUBEMAP: launch2<LMAX, VLB_SKY_CUBEMAP>(a, tma, num_sms, s); break;
    case VLB_SKY_PANORAMA: launch2<LMAX, VLB_SKY_PANORAMA>(a, tma, num_sms, s); break;
    default: launch2<LMAX, VLB_SKY_ENVMAP>(a, tma, num_sms, s); break;
  }
}

int launch_skybox_sh(const SkyboxArgs& a, bool tma, int num_sms, cudaStream_t s) {
  if (tma && a.pair_table && a.layout == VLB_SKY_CUBEMAP) {
    const bool rgb = a.fmt == VLB_TEXEL_RGB32F;
    // measured on 1024 maps of 6 x 128^2 RGB FP32, L2: two maps a warp (16 a
    // basis row, 162 registers, one CTA per SM) 81 % of the HBM copy rate,
    // one map a warp (two CTAs per SM) 77 %
    if (a.lmax == 2) { if (rgb) launch_group<2, 0, 2, 3>(a, num_sms, s); else launch_group<2, 1, 2, 3>(a, num_sms, s); }
    else if (rgb) launch_group<3, 0, 1, 3>(a, num_sms, s);
    else launch_group<3, 1, 1, 3>(a, num_sms, s);
    return int(a.slabs_per_map);  // one partial per (map, slab)
  }
  if (a.lmax == 2) launch1<2>(a, tma, num_sms, s);
  else launch1<3>(a, tma, num_sms, s);
  return int(a.slabs_per_map) * kSkyPartialsPerSlab;
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
