// k_trace.cu -- software ray tracing for the probe bake: the GB300 stand-in
// for the reference's hardware RT pipeline (EnvMapGenerator::getMap,
// src/baker/env_map_generator.cpp:325-359: env_map.rgen -> traversal ->
// env_map.rchit, shadow.rmiss, main.rmiss).
//
// Warp packets.  Every probe casts the same direction set, so a warp takes 32
// spatially close probes (a Morton-sorted packet) and traces direction s for
// all of them at once: 32 parallel rays from nearby origins.  The warp walks
// ONE node stack: each node and triangle is fetched once per warp (a uniform
// address, broadcast to the lanes), every lane tests its own ray, and warp
// ballots decide which children to visit.  All control flow is warp-uniform,
// so no lane idles on a divergent path.  A lane's result is exactly its own
// closest hit -- the warp visits a superset of the nodes the lane needs -- and
// equal distances resolve to the lower triangle index, so results do not
// depend on which probes share the packet.
//
// Per ray:
//   closest hit in (tmin, tmax)                    [env_map.rgen:22-26]
//   hit:  n = geometric normal facing the ray; if n.l > 0 a shadow ray from
//         hit + bias*n toward the sun, any-hit      [env_map.rchit:79-88]
//         radiance = albedo * sun/pi * n.l * lit    (Lambert + directional sun)
//   miss: nearest texel of the cubemap sky, or 0   [main.rmiss:37-41]
// BVH2 nodes hold both children's boxes (4 x float4 = 64 B); triangles are
// 3 x float4 in leaf order.
//
// Fused mode: each lane accumulates its probe's K x 3 coefficients over the
// warp's directions (the basis row is warp-uniform); the CTA's warps are
// consecutive direction chunks of the same packet and are summed in shared
// memory in a fixed order; the last CTA of a packet (atomic ticket) adds the
// CTA partials in FP64 in a fixed order and writes the output.  Tile mode
// writes the [probe][3][S] radiance tile instead (the plain path).
#include <cuda_bf16.h>

#include "vlb_device.cuh"
#include "vlb_internal.h"

namespace vlbk {

constexpr int kTraceThreads = kTraceWarps * 32;
constexpr unsigned kFull = 0xffffffffu;

struct RayCtx {
  float ox, oy, oz, dx, dy, dz;
  float ix, iy, iz;     // 1 / d (zero components nudged to 1e-30)
  float oix, oiy, oiz;  // o * inv
};

struct Work {
  uint32_t wnodes = 0, wtris = 0, shadow = 0, lnodes = 0;
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

// Warp-cooperative traversal.  ANY = false: closest hit in (tmin, tbest)
// with ties to the lower triangle id; ANY = true: a lane stops (active =
// false, best_slot >= 0) at its first hit in (tmin, tbest).  Must be called
// by all 32 lanes; lanes with active == false only vote "no".
template <bool ANY, bool COUNT>
__device__ __forceinline__ void packet_traverse(const RayCtx& r, bool& active, const float4* __restrict__ nodes,
                                                const float4* __restrict__ tris, uint32_t ntris, float tmin,
                                                float& tbest, int& best_slot, int& best_id, int* err, Work& w) {
  if (ntris == 0 || !__any_sync(kFull, active)) return;
  const uint32_t lane = threadIdx.x & 31;
  int stack[kTraceStack];
  int sp = 0;
  int cur = ntris > 1 ? 0 : ~0;
  for (;;) {
    if (cur >= 0) {
      if constexpr (COUNT) { w.wnodes += lane == 0; w.lnodes += active; }
      const float4 n0 = __ldg(nodes + 4 * cur), n1 = __ldg(nodes + 4 * cur + 1), n2 = __ldg(nodes + 4 * cur + 2),
                   n3 = __ldg(nodes + 4 * cur + 3);
      bool h0 = false, h1 = false;
      float tn0 = 0.f, tn1 = 0.f;
      if (active) {
        h0 = slab(r, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, tmin, tbest, &tn0);
        h1 = slab(r, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, tmin, tbest, &tn1);
      }
      const unsigned b0 = __ballot_sync(kFull, h0), b1 = __ballot_sync(kFull, h1);
      const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
      if (b0 && b1) {
        bool first0 = true;
        if constexpr (!ANY) {
          // visit first the child most lanes reach first (efficiency only)
          const unsigned pref0 = __ballot_sync(kFull, h0 && (!h1 || tn0 <= tn1));
          first0 = 2 * __popc(pref0) >= __popc(b0 | b1);
        }
        if (sp < kTraceStack) stack[sp++] = first0 ? c1 : c0;
        else if (lane == 0) atomicAdd(err + kErrStackOverflow, 1);
        cur = first0 ? c0 : c1;
        continue;
      }
      if (b0) { cur = c0; continue; }
      if (b1) { cur = c1; continue; }
    } else {
      if constexpr (COUNT) w.wtris += lane == 0;
      const int slot = ~cur;
      const float4 v0 = __ldg(tris + 3 * slot), e1 = __ldg(tris + 3 * slot + 1), e2 = __ldg(tris + 3 * slot + 2);
      if (active) {
        const float t = tri_hit(r, v0, e1, e2);
        if (t > tmin) {
          if constexpr (ANY) {
            if (t < tbest) { best_slot = slot; active = false; }
          } else {
            const int id = __float_as_int(v0.w);
            if (t < tbest || (t == tbest && best_slot >= 0 && id < best_id)) { tbest = t; best_slot = slot; best_id = id; }
          }
        }
      }
      if constexpr (ANY) {
        if (!__any_sync(kFull, active)) break;
      }
    }
    if (sp == 0) break;
    cur = stack[--sp];
  }
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

// One sample for the whole warp: primary packet, shading, shadow packet.
template <bool COUNT>
__device__ __forceinline__ Shaded trace_sample(const TraceArgs& a, bool valid, float ox, float oy, float oz,
                                               const float4 d, Work& w) {
  RayCtx ray;
  make_ray(ray, ox, oy, oz, d.x, d.y, d.z);
  bool act = valid;
  float tb = a.tmax;
  int slot = -1, id = -1;
  packet_traverse<false, COUNT>(ray, act, a.nodes, a.tris, a.ntris, a.tmin, tb, slot, id, a.err, w);
  Shaded o{0.f, 0.f, 0.f, -1, 2};
  RayCtx sh = ray;
  bool need = false;
  float ndl = 0.f, nx = 0.f, ny = 0.f, nz = 0.f;
  if (valid) {
    if (slot < 0) {
      if (a.sky) {
        const float* tx = a.sky + 3 * size_t(cube_texel(d.x, d.y, d.z, a.sky_n));
        o.r = __ldg(tx); o.g = __ldg(tx + 1); o.b = __ldg(tx + 2);
      }
    } else {
      const float4 e1 = __ldg(a.tris + 3 * slot + 1), e2 = __ldg(a.tris + 3 * slot + 2);
      o.tri = id;
      nx = e1.y * e2.z - e1.z * e2.y; ny = e1.z * e2.x - e1.x * e2.z; nz = e1.x * e2.y - e1.y * e2.x;
      const float rn = rsqrtf(nx * nx + ny * ny + nz * nz);
      nx *= rn; ny *= rn; nz *= rn;
      if (nx * d.x + ny * d.y + nz * d.z > 0.f) { nx = -nx; ny = -ny; nz = -nz; }
      ndl = nx * a.sun.x + ny * a.sun.y + nz * a.sun.z;
      if (ndl > 0.f) {
        need = true;
        make_ray(sh, fmaf(tb, d.x, ox) + a.bias * nx, fmaf(tb, d.y, oy) + a.bias * ny, fmaf(tb, d.z, oz) + a.bias * nz,
                 a.sun.x, a.sun.y, a.sun.z);
      }
    }
  }
  if constexpr (COUNT) w.shadow += need;
  bool sact = need;
  float stb = a.tmax;
  int sslot = -1, sid = -1;
  packet_traverse<true, COUNT>(sh, sact, a.nodes, a.tris, a.ntris, 0.0f, stb, sslot, sid, a.err, w);
  if (need) {
    const bool occ = sslot >= 0;
    o.vis = occ ? 0 : 1;
    if (!occ) {
      const float k = a.sun_scale * ndl;
      const float4 alb = __ldg(a.albedo + o.tri);
      o.r = alb.x * k; o.g = alb.y * k; o.b = alb.z * k;
    }
  }
  return o;
}

template <bool COUNT>
__device__ __forceinline__ void flush_counts(const TraceArgs& a, const Work& w) {
  if constexpr (COUNT) {
    atomicAdd(a.counters + 0, (unsigned long long)w.wnodes);
    atomicAdd(a.counters + 1, (unsigned long long)w.wtris);
    atomicAdd(a.counters + 2, (unsigned long long)w.shadow);
    atomicAdd(a.counters + 3, (unsigned long long)w.lnodes);
  }
}

// Plain path: writes the [probe][3][S] radiance tile (FP32 and/or BF16).
template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads) k_trace_tile(const TraceArgs a) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t pg = blockIdx.x / a.block_chunks, bc = blockIdx.x - pg * a.block_chunks;
  const uint32_t chunk = bc * kTraceWarps + warp;
  const uint32_t slot = pg * 32 + lane;
  const bool valid = slot < a.nprobes;
  const uint32_t p = valid ? (a.order ? a.order[slot] : slot) : 0;
  const float ox = valid ? a.probes[3 * size_t(p)] : 0.f, oy = valid ? a.probes[3 * size_t(p) + 1] : 0.f,
              oz = valid ? a.probes[3 * size_t(p) + 2] : 0.f;
  const uint32_t s0 = min(a.S, chunk * a.dirs_per_warp), s1 = min(a.S, s0 + a.dirs_per_warp);
  Work w;
  for (uint32_t s = s0; s < s1; ++s) {
    const Shaded o = trace_sample<COUNT>(a, valid, ox, oy, oz, __ldg(a.dirs + s), w);
    if (!valid) continue;
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

template <int K>
__global__ void __launch_bounds__(kTraceThreads) k_trace_fused(const TraceArgs a) {
  constexpr int V = 3 * K;
  __shared__ float red[kTraceWarps][32][V + 1];
  __shared__ uint32_t ticket;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t pg = blockIdx.x / a.block_chunks, bc = blockIdx.x - pg * a.block_chunks;
  const uint32_t chunk = bc * kTraceWarps + warp;
  const uint32_t slot = pg * 32 + lane;
  const bool valid = slot < a.nprobes;
  const uint32_t p = valid ? (a.order ? a.order[slot] : slot) : 0;
  const float ox = valid ? a.probes[3 * size_t(p)] : 0.f, oy = valid ? a.probes[3 * size_t(p) + 1] : 0.f,
              oz = valid ? a.probes[3 * size_t(p) + 2] : 0.f;
  const uint32_t s0 = min(a.S, chunk * a.dirs_per_warp), s1 = min(a.S, s0 + a.dirs_per_warp);
  float acc[V];
#pragma unroll
  for (int v = 0; v < V; ++v) acc[v] = 0.f;
  Work w;
  for (uint32_t s = s0; s < s1; ++s) {
    const Shaded o = trace_sample<false>(a, valid, ox, oy, oz, __ldg(a.dirs + s), w);
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
    if (valid) {
      const size_t ri = size_t(p) * a.S + s;
      if (a.hit_tri) a.hit_tri[ri] = o.tri;
      if (a.shadow) a.shadow[ri] = o.vis;
    }
  }
  // CTA reduction over its warps (consecutive direction chunks), fixed order
#pragma unroll
  for (int v = 0; v < V; ++v) red[warp][lane][v] = acc[v];
  __syncthreads();
  const bool direct = a.block_chunks == 1;
  for (uint32_t e = threadIdx.x; e < 32u * V; e += kTraceThreads) {
    const uint32_t l = e / V, v = e - l * V;
    const uint32_t sl = pg * 32 + l;
    if (sl >= a.nprobes) continue;
    float s = 0.f;
#pragma unroll
    for (int wi = 0; wi < kTraceWarps; ++wi) s += red[wi][l][v];
    const uint32_t pp = a.order ? a.order[sl] : sl;
    if (direct) a.out[size_t(pp) * V + v] = s;
    else a.partial[(size_t(pp) * a.block_chunks + bc) * V + v] = s;
  }
  if (direct) return;
  // the last CTA of this packet sums the CTA partials in FP64, fixed order
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(a.group_done + pg, 1u);
  __syncthreads();
  if (ticket != a.block_chunks - 1) return;
  __threadfence();
  for (uint32_t e = threadIdx.x; e < 32u * V; e += kTraceThreads) {
    const uint32_t l = e / V, v = e - l * V;
    const uint32_t sl = pg * 32 + l;
    if (sl >= a.nprobes) continue;
    const uint32_t pp = a.order ? a.order[sl] : sl;
    const float* src = a.partial + size_t(pp) * a.block_chunks * V + v;
    double s = 0.0;
    for (uint32_t j = 0; j < a.block_chunks; ++j) s += double(__ldcg(src + size_t(j) * V));
    a.out[size_t(pp) * V + v] = float(s);
  }
}

void plan_trace(TraceArgs& a, int num_sms) {
  const uint64_t npg = (uint64_t(a.nprobes) + 31) / 32;
  const uint64_t target = uint64_t(num_sms) * 48;  // warps
  uint64_t nsc = (target + npg - 1) / npg;
  uint64_t bcn = (nsc + kTraceWarps - 1) / kTraceWarps;
  nsc = bcn * kTraceWarps;
  uint64_t dpw = (a.S + nsc - 1) / nsc;
  if (dpw == 0) dpw = 1;
  const uint64_t nsc_eff = (a.S + dpw - 1) / dpw;
  bcn = (nsc_eff + kTraceWarps - 1) / kTraceWarps;
  a.dirs_per_warp = uint32_t(dpw);
  a.block_chunks = uint32_t(bcn > 0 ? bcn : 1);
}

static uint32_t trace_grid(const TraceArgs& a) {
  return uint32_t(((uint64_t(a.nprobes) + 31) / 32) * a.block_chunks);
}

void launch_trace_tile(const TraceArgs& a, cudaStream_t s) {
  const uint32_t g = trace_grid(a);
  if (!g) return;
  if (a.counters) k_trace_tile<true><<<g, kTraceThreads, 0, s>>>(a);
  else k_trace_tile<false><<<g, kTraceThreads, 0, s>>>(a);
}

void launch_trace_fused(const TraceArgs& a, cudaStream_t s) {
  const uint32_t g = trace_grid(a);
  if (!g) return;
  if (a.K == 9) k_trace_fused<9><<<g, kTraceThreads, 0, s>>>(a);
  else k_trace_fused<16><<<g, kTraceThreads, 0, s>>>(a);
}

}  // namespace vlbk
