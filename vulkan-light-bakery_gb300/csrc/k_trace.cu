// k_trace.cu -- software ray tracing for the probe bake: the GB300 stand-in
// for the reference's hardware RT pipeline (EnvMapGenerator::getMap,
// src/baker/env_map_generator.cpp:325-359: env_map.rgen -> traversal ->
// env_map.rchit, shadow.rmiss, main.rmiss).
//
// Thread mapping: a warp is 32 probes (consecutive in the caller's order)
// tracing the SAME sample direction at the same time, so the 32 rays are
// parallel and start close together and walk nearly the same BVH nodes; each
// warp loops over a chunk of directions.  Per ray:
//   closest hit in (tmin, tmax)                    [env_map.rgen:22-26]
//   hit:  n = geometric normal facing the ray; if n.l > 0 a shadow ray from
//         hit + bias*n toward the sun, any-hit      [env_map.rchit:79-88]
//         radiance = albedo * sun/pi * n.l * lit    (Lambert + directional sun)
//   miss: nearest texel of the cubemap sky, or 0   [main.rmiss:37-41]
// BVH2 nodes hold both children's boxes (4 x float4 = 64 B, one coalesced
// fetch per node); triangles are 3 x float4 in leaf order.  The traversal
// stack lives in local memory (L1); overflow bumps an error counter.
// The COUNT instantiations tally nodes fetched and triangles tested per ray
// (the algorithmic bytes of the traversal); the timed kernels compile
// without them.
#include <cuda_bf16.h>

#include "vlb_device.cuh"
#include "vlb_internal.h"

namespace vlbk {

constexpr int kTraceThreads = 128;

struct RayCtx {
  float ox, oy, oz, dx, dy, dz;
  float ix, iy, iz;     // 1 / d (zero components nudged to 1e-30)
  float oix, oiy, oiz;  // o * inv
};

struct Work {
  uint32_t nodes = 0, tris = 0, shadow = 0;
};

__device__ __forceinline__ float safe_inv(float d) {
  return 1.0f / (fabsf(d) > 1e-30f ? d : copysignf(1e-30f, d));
}

__device__ __forceinline__ void make_ray(RayCtx& r, float ox, float oy, float oz, float dx, float dy, float dz) {
  r.ox = ox; r.oy = oy; r.oz = oz; r.dx = dx; r.dy = dy; r.dz = dz;
  r.ix = safe_inv(dx); r.iy = safe_inv(dy); r.iz = safe_inv(dz);
  r.oix = ox * r.ix; r.oiy = oy * r.iy; r.oiz = oz * r.iz;
}

__device__ __forceinline__ bool slab(const RayCtx& r, float lx, float ly, float lz, float hx, float hy, float hz,
                                     float tmin, float tmax, float* tnear) {
  const float t0x = fmaf(lx, r.ix, -r.oix), t1x = fmaf(hx, r.ix, -r.oix);
  const float t0y = fmaf(ly, r.iy, -r.oiy), t1y = fmaf(hy, r.iy, -r.oiy);
  const float t0z = fmaf(lz, r.iz, -r.oiz), t1z = fmaf(hz, r.iz, -r.oiz);
  const float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
  const float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax));
  *tnear = tn;
  return tn <= tf;
}

// Moller-Trumbore, inclusive edges; returns t or -1.
__device__ __forceinline__ float tri_hit(const RayCtx& r, const float4 v0, const float4 e1, const float4 e2) {
  const float px = r.dy * e2.z - r.dz * e2.y, py = r.dz * e2.x - r.dx * e2.z, pz = r.dx * e2.y - r.dy * e2.x;
  const float det = e1.x * px + e1.y * py + e1.z * pz;
  if (det == 0.f) return -1.f;
  const float inv = 1.0f / det;
  const float sx = r.ox - v0.x, sy = r.oy - v0.y, sz = r.oz - v0.z;
  const float u = (sx * px + sy * py + sz * pz) * inv;
  if (u < 0.f || u > 1.f) return -1.f;
  const float qx = sy * e1.z - sz * e1.y, qy = sz * e1.x - sx * e1.z, qz = sx * e1.y - sy * e1.x;
  const float v = (r.dx * qx + r.dy * qy + r.dz * qz) * inv;
  if (v < 0.f || u + v > 1.f) return -1.f;
  return (e2.x * qx + e2.y * qy + e2.z * qz) * inv;
}

// Closest hit (ANY = false) or first hit (ANY = true) in (tmin, tmax).
// Returns the leaf slot or -1; *t_out = hit distance for closest hit.
template <bool ANY, bool COUNT>
__device__ int traverse(const RayCtx& r, const float4* __restrict__ nodes, const float4* __restrict__ tris,
                        uint32_t ntris, float tmin, float tmax, float* t_out, int* err, Work& w) {
  if (ntris == 0) return -1;
  int stack[kTraceStack];
  int sp = 0;
  int cur = ntris > 1 ? 0 : ~0;
  float tbest = tmax;
  int best = -1;
  for (;;) {
    if (cur >= 0) {
      if constexpr (COUNT) ++w.nodes;
      const float4 n0 = __ldg(nodes + 4 * cur), n1 = __ldg(nodes + 4 * cur + 1), n2 = __ldg(nodes + 4 * cur + 2),
                   n3 = __ldg(nodes + 4 * cur + 3);
      float tn0, tn1;
      const bool h0 = slab(r, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, tmin, tbest, &tn0);
      const bool h1 = slab(r, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, tmin, tbest, &tn1);
      const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
      if (h0 && h1) {
        const bool first0 = ANY || tn0 <= tn1;
        if (sp < kTraceStack) stack[sp++] = first0 ? c1 : c0;
        else atomicAdd(err + kErrStackOverflow, 1);
        cur = first0 ? c0 : c1;
        continue;
      }
      if (h0) { cur = c0; continue; }
      if (h1) { cur = c1; continue; }
    } else {
      if constexpr (COUNT) ++w.tris;
      const int slot = ~cur;
      const float4 v0 = __ldg(tris + 3 * slot), e1 = __ldg(tris + 3 * slot + 1), e2 = __ldg(tris + 3 * slot + 2);
      const float t = tri_hit(r, v0, e1, e2);
      if (t > tmin && t < tbest) {
        if constexpr (ANY) return slot;
        tbest = t;
        best = slot;
      }
    }
    if (sp == 0) break;
    cur = stack[--sp];
  }
  *t_out = tbest;
  return best;
}

// Nearest cubemap texel; each step one IEEE FP32 operation (matches the
// oracle's texel choice exactly).
__device__ __forceinline__ uint32_t cube_texel(float x, float y, float z, uint32_t n) {
  const float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
  float sc, tc, ma;
  uint32_t f;
  if (ax >= ay && ax >= az) {
    if (x >= 0.f) { f = 0; sc = -z; tc = -y; } else { f = 1; sc = z; tc = -y; }
    ma = ax;
  } else if (ay >= az) {
    if (y >= 0.f) { f = 2; sc = x; tc = z; } else { f = 3; sc = x; tc = -z; }
    ma = ay;
  } else {
    if (z >= 0.f) { f = 4; sc = x; tc = -y; } else { f = 5; sc = -x; tc = -y; }
    ma = az;
  }
  const float fn = float(n);
  const float fu = __fmul_rn(__fmul_rn(__fadd_rn(__fdiv_rn(sc, ma), 1.0f), 0.5f), fn);
  const float fv = __fmul_rn(__fmul_rn(__fadd_rn(__fdiv_rn(tc, ma), 1.0f), 0.5f), fn);
  const int ix = min(max(int(floorf(fu)), 0), int(n) - 1);
  const int iy = min(max(int(floorf(fv)), 0), int(n) - 1);
  return (f * n + uint32_t(iy)) * n + uint32_t(ix);
}

struct Shaded {
  float r, g, b;
  int tri;      // original triangle id or -1
  uint8_t vis;  // 0 occluded, 1 lit, 2 no shadow ray
};

template <bool COUNT>
__device__ __forceinline__ Shaded shade(const TraceArgs& a, const RayCtx& ray, Work& w) {
  Shaded o;
  float t;
  const int slot = traverse<false, COUNT>(ray, a.nodes, a.tris, a.ntris, a.tmin, a.tmax, &t, a.err, w);
  if (slot < 0) {
    o.tri = -1; o.vis = 2;
    if (a.sky) {
      const float* tx = a.sky + 3 * size_t(cube_texel(ray.dx, ray.dy, ray.dz, a.sky_n));
      o.r = __ldg(tx); o.g = __ldg(tx + 1); o.b = __ldg(tx + 2);
    } else {
      o.r = o.g = o.b = 0.f;
    }
    return o;
  }
  const float4 v0 = __ldg(a.tris + 3 * slot), e1 = __ldg(a.tris + 3 * slot + 1), e2 = __ldg(a.tris + 3 * slot + 2);
  o.tri = __float_as_int(v0.w);
  float nx = e1.y * e2.z - e1.z * e2.y, ny = e1.z * e2.x - e1.x * e2.z, nz = e1.x * e2.y - e1.y * e2.x;
  const float rn = rsqrtf(nx * nx + ny * ny + nz * nz);
  nx *= rn; ny *= rn; nz *= rn;
  if (nx * ray.dx + ny * ray.dy + nz * ray.dz > 0.f) { nx = -nx; ny = -ny; nz = -nz; }
  const float ndl = nx * a.sun.x + ny * a.sun.y + nz * a.sun.z;
  if (!(ndl > 0.f)) { o.r = o.g = o.b = 0.f; o.vis = 2; return o; }
  RayCtx sh;
  make_ray(sh, fmaf(t, ray.dx, ray.ox) + a.bias * nx, fmaf(t, ray.dy, ray.oy) + a.bias * ny,
           fmaf(t, ray.dz, ray.oz) + a.bias * nz, a.sun.x, a.sun.y, a.sun.z);
  if constexpr (COUNT) ++w.shadow;
  float ts;
  const bool occ = traverse<true, COUNT>(sh, a.nodes, a.tris, a.ntris, 0.0f, a.tmax, &ts, a.err, w) >= 0;
  o.vis = occ ? 0 : 1;
  const float k = occ ? 0.f : a.sun_scale * ndl;
  const float4 alb = __ldg(a.albedo + o.tri);
  o.r = alb.x * k; o.g = alb.y * k; o.b = alb.z * k;
  return o;
}

template <bool COUNT>
__device__ __forceinline__ void flush_counts(const TraceArgs& a, const Work& w) {
  if constexpr (COUNT) {
    atomicAdd(a.counters + 0, uint64_t(w.nodes));
    atomicAdd(a.counters + 1, uint64_t(w.tris));
    atomicAdd(a.counters + 2, uint64_t(w.shadow));
  }
}

// Plain path: writes the [probe][3][S] radiance tile (FP32 and/or BF16).
template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads) k_trace_tile(const TraceArgs a) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gw = blockIdx.x * (kTraceThreads / 32) + (threadIdx.x >> 5);
  const uint32_t nsc = (a.S + a.dirs_per_warp - 1) / a.dirs_per_warp;
  const uint32_t pg = gw / nsc, sc = gw - pg * nsc;
  const uint32_t p = pg * 32 + lane;
  if (p >= a.nprobes) return;
  const float ox = a.probes[3 * size_t(p)], oy = a.probes[3 * size_t(p) + 1], oz = a.probes[3 * size_t(p) + 2];
  const uint32_t s0 = sc * a.dirs_per_warp, s1 = min(a.S, s0 + a.dirs_per_warp);
  Work w;
  for (uint32_t s = s0; s < s1; ++s) {
    const float4 d = __ldg(a.dirs + s);
    RayCtx ray;
    make_ray(ray, ox, oy, oz, d.x, d.y, d.z);
    const Shaded o = shade<COUNT>(a, ray, w);
    const size_t row = size_t(p) * 3;
    if (a.radiance) {
      a.radiance[row * a.S + s] = o.r;
      a.radiance[(row + 1) * a.S + s] = o.g;
      a.radiance[(row + 2) * a.S + s] = o.b;
    }
    if (a.radiance_bf16) {
      a.radiance_bf16[row * a.S + s] = __bfloat16_as_ushort(__float2bfloat16_rn(o.r));
      a.radiance_bf16[(row + 1) * a.S + s] = __bfloat16_as_ushort(__float2bfloat16_rn(o.g));
      a.radiance_bf16[(row + 2) * a.S + s] = __bfloat16_as_ushort(__float2bfloat16_rn(o.b));
    }
    const size_t ri = size_t(p) * a.S + s;
    if (a.hit_tri) a.hit_tri[ri] = o.tri;
    if (a.shadow) a.shadow[ri] = o.vis;
    if (a.dbg_radiance) {
      a.dbg_radiance[3 * ri] = o.r; a.dbg_radiance[3 * ri + 1] = o.g; a.dbg_radiance[3 * ri + 2] = o.b;
    }
  }
  flush_counts<COUNT>(a, w);
}

// Fused path: each lane accumulates its probe's K x 3 coefficients over its
// chunk of directions (the basis row is the same for the whole warp, a
// broadcast load) and writes one partial per (probe, chunk).
template <int K>
__global__ void __launch_bounds__(kTraceThreads) k_trace_fused(const TraceArgs a) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gw = blockIdx.x * (kTraceThreads / 32) + (threadIdx.x >> 5);
  const uint32_t nsc = (a.S + a.dirs_per_warp - 1) / a.dirs_per_warp;
  const uint32_t pg = gw / nsc, sc = gw - pg * nsc;
  const uint32_t p = pg * 32 + lane;
  if (p >= a.nprobes) return;
  const float ox = a.probes[3 * size_t(p)], oy = a.probes[3 * size_t(p) + 1], oz = a.probes[3 * size_t(p) + 2];
  const uint32_t s0 = sc * a.dirs_per_warp, s1 = min(a.S, s0 + a.dirs_per_warp);
  float acc[3 * K];
#pragma unroll
  for (int v = 0; v < 3 * K; ++v) acc[v] = 0.f;
  Work w;
  for (uint32_t s = s0; s < s1; ++s) {
    const float4 d = __ldg(a.dirs + s);
    RayCtx ray;
    make_ray(ray, ox, oy, oz, d.x, d.y, d.z);
    const Shaded o = shade<false>(a, ray, w);
    const float4* b4 = reinterpret_cast<const float4*>(a.basis16 + size_t(s) * 16);
#pragma unroll
    for (int q = 0; q < (K + 3) / 4; ++q) {
      const float4 b = __ldg(b4 + q);
      const float bb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int k = 4 * q + e;
        if (k < K) {
          acc[3 * k] = fmaf(bb[e], o.r, acc[3 * k]);
          acc[3 * k + 1] = fmaf(bb[e], o.g, acc[3 * k + 1]);
          acc[3 * k + 2] = fmaf(bb[e], o.b, acc[3 * k + 2]);
        }
      }
    }
    const size_t ri = size_t(p) * a.S + s;
    if (a.hit_tri) a.hit_tri[ri] = o.tri;
    if (a.shadow) a.shadow[ri] = o.vis;
  }
  float* out = a.partial + (size_t(p) * nsc + sc) * (3 * K);
#pragma unroll
  for (int v = 0; v < 3 * K; ++v) out[v] = acc[v];
}

static uint32_t trace_grid(const TraceArgs& a) {
  const uint32_t nsc = (a.S + a.dirs_per_warp - 1) / a.dirs_per_warp;
  const uint64_t warps = uint64_t((a.nprobes + 31) / 32) * nsc;
  return uint32_t((warps + kTraceThreads / 32 - 1) / (kTraceThreads / 32));
}

void launch_trace_tile(const TraceArgs& a, cudaStream_t s) {
  const uint32_t g = trace_grid(a);
  if (!g) return;
  if (a.counters) k_trace_tile<true><<<g, kTraceThreads, 0, s>>>(a);
  else k_trace_tile<false><<<g, kTraceThreads, 0, s>>>(a);
}

void launch_trace_fused(const TraceArgs& a, cudaStream_t s, uint32_t* chunks_out) {
  const uint32_t g = trace_grid(a);
  if (chunks_out) *chunks_out = (a.S + a.dirs_per_warp - 1) / a.dirs_per_warp;
  if (!g) return;
  if (a.K == 9) k_trace_fused<9><<<g, kTraceThreads, 0, s>>>(a);
  else k_trace_fused<16><<<g, kTraceThreads, 0, s>>>(a);
}

}  // namespace vlbk
