// trace_common.cuh -- device pieces shared by the trace kernels (k_trace.cu,
// k_trace_fused.cu): ray setup, box and triangle tests, the packet and
// per-lane BVH walks, shading of a primary hit, and the per-lane ray state
// machine of the lane walks.  See k_trace.cu for the traversal rules (the
// pruning margin, the tie rule) that make every ray's result independent of
// the walk that finds it.
#pragma once

#include <cuda_bf16.h>

#include <climits>

#include "vlb_device.cuh"
#include "vlb_internal.h"

namespace vlbk {
constexpr int kTraceThreads = kTraceWarps * 32;
constexpr unsigned kFull = 0xffffffffu;

// The box-test terms as pairs for packed FMAs: a plane p of axis a is crossed
// at t = p * inv_a - o_a * inv_a, i.e. fma(p, inv_a, -(o_a * inv_a)).
struct RayCtx {
  float ox, oy, oz, dx, dy, dz;
  float2 ixy, izz;  // (1/dx, 1/dy), (1/dz, 1/dz) (zero components nudged to 1e-30)
  float2 nxy, nzz;  // -(o * inv) for the same components
};

struct Work {
  uint32_t wnodes = 0, wtris = 0, shadow = 0, lnodes = 0;
};

__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

__device__ __forceinline__ float safe_inv(float d) {
  return 1.0f / (fabsf(d) > 1e-30f ? d : copysignf(1e-30f, d));
}

__device__ __forceinline__ void make_ray_inv(RayCtx& r, float ox, float oy, float oz, float dx, float dy, float dz,
                                             float ix, float iy, float iz) {
  r.ox = ox; r.oy = oy; r.oz = oz; r.dx = dx; r.dy = dy; r.dz = dz;
  const float nz = -(oz * iz);
  r.ixy = make_float2(ix, iy);
  r.izz = make_float2(iz, iz);
  r.nxy = make_float2(-(ox * ix), -(oy * iy));
  r.nzz = make_float2(nz, nz);
}

__device__ __forceinline__ void make_ray(RayCtx& r, float ox, float oy, float oz, float dx, float dy, float dz) {
  make_ray_inv(r, ox, oy, oz, dx, dy, dz, safe_inv(dx), safe_inv(dy), safe_inv(dz));
}

// (a.x * b.x + c.x, a.y * b.y + c.y), each one fma.rn.f32 (one packed instruction).
__device__ __forceinline__ float2 fma_pair(float ax, float ay, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 a, b, c, d;\n\t"
      "mov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\tmov.b64 c, {%6, %7};\n\t"
      "fma.rn.f32x2 d, a, b, c;\n\tmov.b64 {%0, %1}, d;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(ax), "f"(ay), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}

// make_ray with the reciprocals of d precomputed (host_safe_inv: the same bits).
// Slab test for a ray in octant OCT (bit a set: 1/d_a < 0).  The octant is
// the same for every lane of a packet (one direction per packet), so the
// entry and exit planes of each axis are chosen at compile time and no
// per-axis min/max is needed.
template <int OCT>
__device__ __forceinline__ bool slab(const RayCtx& r, float lx, float ly, float lz, float hx, float hy, float hz,
                                     float tmin, float tmax, float* tnear) {
  const float ix = r.ixy.x, iy = r.ixy.y, iz = r.izz.x, nx = r.nxy.x, ny = r.nxy.y, nz = r.nzz.x;
  const float tnx = fmaf((OCT & 1) ? hx : lx, ix, nx), tfx = fmaf((OCT & 1) ? lx : hx, ix, nx);
  const float tny = fmaf((OCT & 2) ? hy : ly, iy, ny), tfy = fmaf((OCT & 2) ? ly : hy, iy, ny);
  const float tnz = fmaf((OCT & 4) ? hz : lz, iz, nz), tfz = fmaf((OCT & 4) ? lz : hz, iz, nz);
  const float tn = fmax3(tnx, tny, fmaxf(tnz, tmin));
  const float tf = fmin3(tfx, tfy, fminf(tfz, tmax));
  *tnear = tn;
  return tn <= tf;
}

__device__ __forceinline__ int octant_of(float dx, float dy, float dz) {
  return (safe_inv(dx) < 0.f ? 1 : 0) | (safe_inv(dy) < 0.f ? 2 : 0) | (safe_inv(dz) < 0.f ? 4 : 0);
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

// One 64-byte node as two 256-bit read-only loads (a node starts on a 64-byte
// boundary): half the load instructions of four 128-bit loads.
__device__ __forceinline__ void ldg_node(const float4* p, float4& n0, float4& n1, float4& n2, float4& n3) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(n0.x), "=f"(n0.y), "=f"(n0.z), "=f"(n0.w), "=f"(n1.x), "=f"(n1.y), "=f"(n1.z), "=f"(n1.w)
      : "l"(p));
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(n2.x), "=f"(n2.y), "=f"(n2.z), "=f"(n2.w), "=f"(n3.x), "=f"(n3.y), "=f"(n3.z), "=f"(n3.w)
      : "l"(p + 2));
}

// Far limit of the box tests: the best distance so far plus a relative 2^-12.
__device__ __forceinline__ float prune_limit(float tbest) { return fmaf(tbest, 0x1p-12f, tbest); }

// Warp-uniform stack of up to kTraceStack (64) node references held in two
// registers per lane: entry i sits in lane i % 32, register i / 32, together
// with the ballot of the lanes whose own box test accepted that subtree.
struct WarpStack {
  int r0 = 0, r1 = 0, sp = 0;
  unsigned m0 = 0, m1 = 0;
  __device__ __forceinline__ void push(int v, unsigned lanes, uint32_t lane, int* err) {
    if (sp >= kTraceStack) {
      if (lane == 0) atomicAdd(err + kErrStackOverflow, 1);
      return;
    }
    if (lane == uint32_t(sp & 31)) {
      if (sp < 32) { r0 = v; m0 = lanes; } else { r1 = v; m1 = lanes; }
    }
    ++sp;
  }
  __device__ __forceinline__ int pop(bool& mine, uint32_t lane) {
    --sp;
    const bool lo = sp < 32;
    const int v = __shfl_sync(kFull, lo ? r0 : r1, sp & 31);
    const unsigned m = __shfl_sync(kFull, lo ? m0 : m1, sp & 31);
    mine = (m >> lane) & 1u;
    return v;
  }
};

// Warp-cooperative traversal.  ANY = false: closest hit in (tmin, tbest)
// with ties to the lower triangle id; ANY = true: a lane stops (active =
// false, best_slot >= 0) at its first hit in (tmin, tbest).  Must be called
// by all 32 lanes; lanes with active == false only vote "no".  OCT is the
// packet's (warp-uniform) ray octant.  A lane tests a node or triangle only
// inside subtrees its own box tests accepted (`in`), so it visits exactly the
// nodes its own walk would, in the warp's order: its result does not depend
// on the other rays of the packet.
template <int OCT, bool ANY, bool COUNT>
__device__ __forceinline__ void packet_traverse(const RayCtx& r, bool& active, const float4* __restrict__ nodes,
                                                const float4* __restrict__ tris, uint32_t ntris, float tmin,
                                                float& tbest, int& best_slot, int& best_id, int* err, Work& w) {
  if (ntris == 0 || !__any_sync(kFull, active)) return;
  const uint32_t lane = threadIdx.x & 31;
  WarpStack st;
  int cur = ntris > 1 ? 0 : ~0;
  bool in = true;
  for (;;) {
    const bool test = active && in;
    if (cur >= 0) {
      if (!VLB_INB(cur, 2 * ntris - 2, err)) break;  // the sibling-pair layout's slots
      if constexpr (COUNT) { w.wnodes += lane == 0; w.lnodes += test; }
      const float4 n0 = __ldg(nodes + 4 * cur), n1 = __ldg(nodes + 4 * cur + 1), n2 = __ldg(nodes + 4 * cur + 2),
                   n3 = __ldg(nodes + 4 * cur + 3);
      bool h0 = false, h1 = false;
      float tn0 = 0.f, tn1 = 0.f;
      if (test) {
        const float lim = prune_limit(tbest);
        h0 = slab<OCT>(r, n0.x, n0.y, n2.x, n0.z, n0.w, n2.y, tmin, lim, &tn0);
        h1 = slab<OCT>(r, n1.x, n1.y, n2.z, n1.z, n1.w, n2.w, tmin, lim, &tn1);
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
        st.push(first0 ? c1 : c0, first0 ? b1 : b0, lane, err);
        cur = first0 ? c0 : c1;
        in = first0 ? h0 : h1;
        continue;
      }
      if (b0) { cur = c0; in = h0; continue; }
      if (b1) { cur = c1; in = h1; continue; }
    } else {
      if constexpr (COUNT) w.wtris += lane == 0;
      const int slot = VLB_CLAMP(~cur, ntris, err);
      const float4 v0 = __ldg(tris + 3 * slot), e1 = __ldg(tris + 3 * slot + 1), e2 = __ldg(tris + 3 * slot + 2);
      if (test) {
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
    if (st.sp == 0) break;
    cur = st.pop(in, lane);
  }
}

// Per-lane traversal (lane mode): the same tests and tie rule as the packet
// walk, the lane's own stack (local memory), nearer child first.  Lanes with
// active == false return at once; no warp collectives.
template <int OCT, bool ANY, bool COUNT>
__device__ __forceinline__ void lane_traverse(const RayCtx& r, bool& active, const float4* __restrict__ nodes,
                                              const float4* __restrict__ tris, uint32_t ntris, float tmin,
                                              float& tbest, int& best_slot, int& best_id, int* err, Work& w) {
  if (ntris == 0 || !active) return;
  int stack[kTraceStack];
  int sp = 0;
  int cur = ntris > 1 ? 0 : ~0;
  for (;;) {
    if (cur >= 0) {
      if (!VLB_INB(cur, 2 * ntris - 2, err)) break;  // the sibling-pair layout's slots
      if constexpr (COUNT) { ++w.wnodes; ++w.lnodes; }
      float4 n0, n1, n2, n3;
      ldg_node(nodes + 4 * cur, n0, n1, n2, n3);
      float tn0, tn1;
      const float lim = prune_limit(tbest);
      const bool h0 = slab<OCT>(r, n0.x, n0.y, n2.x, n0.z, n0.w, n2.y, tmin, lim, &tn0);
      const bool h1 = slab<OCT>(r, n1.x, n1.y, n2.z, n1.z, n1.w, n2.w, tmin, lim, &tn1);
      const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
      if (h0 && h1) {
        const bool first0 = tn0 <= tn1;
        if (sp < kTraceStack) stack[sp++] = first0 ? c1 : c0;
        else atomicAdd(err + kErrStackOverflow, 1);
        cur = first0 ? c0 : c1;
        continue;
      }
      if (h0) { cur = c0; continue; }
      if (h1) { cur = c1; continue; }
    } else {
      if constexpr (COUNT) ++w.wtris;
      const int slot = VLB_CLAMP(~cur, ntris, err);
      const float4 v0 = __ldg(tris + 3 * slot), e1 = __ldg(tris + 3 * slot + 1), e2 = __ldg(tris + 3 * slot + 2);
      const float t = tri_hit(r, v0, e1, e2);
      if (t > tmin) {
        if constexpr (ANY) {
          if (t < tbest) { best_slot = slot; active = false; return; }
        } else {
          const int id = __float_as_int(v0.w);
          if (t < tbest || (t == tbest && best_slot >= 0 && id < best_id)) { tbest = t; best_slot = slot; best_id = id; }
        }
      }
    }
    if (sp == 0) break;
    cur = stack[--sp];
  }
}

// Dispatch on the packet's octant (a warp-uniform branch) and the mode.
template <bool ANY, bool COUNT, bool LANE>
__device__ __forceinline__ void traverse(int oct, const RayCtx& r, bool& active, const float4* __restrict__ nodes,
                                         const float4* __restrict__ tris, uint32_t ntris, float tmin, float& tbest,
                                         int& best_slot, int& best_id, int* err, Work& w) {
#define VLB_OCT(o)                                                                                                \
  case o:                                                                                                         \
    if constexpr (LANE) lane_traverse<o, ANY, COUNT>(r, active, nodes, tris, ntris, tmin, tbest, best_slot,       \
                                                     best_id, err, w);                                            \
    else packet_traverse<o, ANY, COUNT>(r, active, nodes, tris, ntris, tmin, tbest, best_slot, best_id, err, w); \
    break;
  switch (oct) {
    VLB_OCT(0) VLB_OCT(1) VLB_OCT(2) VLB_OCT(3) VLB_OCT(4) VLB_OCT(5) VLB_OCT(6) VLB_OCT(7)
  }
#undef VLB_OCT
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

// One radiance sample into a BF16 tile row.  Plain: [rows][S], the BF16
// rounding of v.  Split (hi/lo): [rows][2S], the rounding hi at column s and
// the rounding of the remainder v - hi at column S + s; hi + lo carries ~16
// mantissa bits of v.
__device__ __forceinline__ void store_bf16(uint16_t* __restrict__ t, size_t row, uint32_t S, uint32_t s, float v,
                                           uint32_t split) {
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  if (!split) {
    t[row * S + s] = __bfloat16_as_ushort(hi);
    return;
  }
  const size_t r0 = row * 2 * size_t(S);
  t[r0 + s] = __bfloat16_as_ushort(hi);
  t[r0 + S + s] = __bfloat16_as_ushort(__float2bfloat16_rn(v - __bfloat162float(hi)));
}

struct Shaded {
  float r, g, b;
  int tri;      // original triangle id or -1
  uint8_t vis;  // 0 occluded, 1 lit, 2 no shadow ray
};

// One sample for the whole warp: primary packet, shading, shadow packet.
// A: any type with the scene and shading fields of TraceArgs (nodes, tris,
// albedo, ntris, tmin, tmax, bias, sun, sun_scale, sky, sky_n, err).
// Primary ray: closest hit -> (slot, id, t); slot -1 on a miss.
template <bool COUNT, bool LANE, class A>
__device__ __forceinline__ void primary_hit(const A& a, bool valid, const RayCtx& ray, const float4 d, int& slot,
                                            int& id, float& tb, Work& w) {
  bool act = valid;
  tb = a.tmax;
  slot = -1;
  id = -1;
  traverse<false, COUNT, LANE>(octant_of(d.x, d.y, d.z), ray, act, a.nodes, a.tris, a.ntris, a.tmin, tb, slot, id,
                               a.err, w);
}

// Shading of a primary result: sky on a miss; at a hit the sun shadow ray
// (any hit) and Lambert.  Called by all 32 lanes (the shadow walk may be a
// packet walk).
template <bool COUNT, bool LANE, class A>
__device__ __forceinline__ Shaded shade_hit(const A& a, bool valid, const RayCtx& ray, float ox, float oy, float oz,
                                            const float4 d, int slot, int id, float tb, Work& w) {
  Shaded o{0.f, 0.f, 0.f, -1, 2};
  RayCtx sh = ray;
  bool need = false;
  float ndl = 0.f;
  if (valid) {
    if (slot < 0) {
      if (a.sky) {
        const float* tx = a.sky + 3 * size_t(VLB_CLAMP(cube_texel(d.x, d.y, d.z, a.sky_n), 6u * a.sky_n * a.sky_n,
                                                       a.err));
        o.r = __ldg(tx); o.g = __ldg(tx + 1); o.b = __ldg(tx + 2);
      }
    } else {
      slot = VLB_CLAMP(slot, a.ntris, a.err);
      const float4 e1 = __ldg(a.tris + 3 * slot + 1), e2 = __ldg(a.tris + 3 * slot + 2);
      o.tri = id;
      float nx = e1.y * e2.z - e1.z * e2.y, ny = e1.z * e2.x - e1.x * e2.z, nz = e1.x * e2.y - e1.y * e2.x;
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
  // inactive lanes keep their primary ray: the octant comes from the sun, uniform
  traverse<true, COUNT, LANE>(octant_of(a.sun.x, a.sun.y, a.sun.z), sh, sact, a.nodes, a.tris, a.ntris, 0.0f, stb,
                              sslot, sid, a.err, w);
  if (need) {
    const bool occ = sslot >= 0;
    o.vis = occ ? 0 : 1;
    if (!occ) {
      const float k = a.sun_scale * ndl;
      const float4 alb = __ldg(a.albedo + VLB_CLAMP(o.tri, a.ntris, a.err));
      o.r = alb.x * k; o.g = alb.y * k; o.b = alb.z * k;
    }
  }
  return o;
}

// One sample for the whole warp: primary walk, shading, shadow walk.
// A: any type with the scene and shading fields of TraceArgs (nodes, tris,
// albedo, ntris, tmin, tmax, bias, sun, sun_scale, sky, sky_n, err).
template <bool COUNT, bool LANE, class A>
__device__ __forceinline__ Shaded trace_sample(const A& a, bool valid, float ox, float oy, float oz, const float4 d,
                                               Work& w) {
  RayCtx ray;
  make_ray(ray, ox, oy, oz, d.x, d.y, d.z);
  int slot, id;
  float tb;
  primary_hit<COUNT, LANE>(a, valid, ray, d, slot, id, tb, w);
  return shade_hit<COUNT, LANE>(a, valid, ray, ox, oy, oz, d, slot, id, tb, w);
}


// ---- per-lane ray state machine (the lane walks) ------------------------------------
// Box test with the octant taken per lane at run time (the lane walks mix
// directions within a warp).
__device__ __forceinline__ bool slab_rt(const RayCtx& r, float lx, float ly, float lz, float hx, float hy, float hz,
                                        float tmin, float tmax, float* tnear) {
  const float ix = r.ixy.x, iy = r.ixy.y, iz = r.izz.x, nx = r.nxy.x, ny = r.nxy.y, nz = r.nzz.x;
  const float ax = fmaf(lx, ix, nx), bx = fmaf(hx, ix, nx);
  const float ay = fmaf(ly, iy, ny), by = fmaf(hy, iy, ny);
  const float az = fmaf(lz, iz, nz), bz = fmaf(hz, iz, nz);
  const float tn = fmax3(fminf(ax, bx), fminf(ay, by), fmaxf(fminf(az, bz), tmin));
  const float tf = fmin3(fmaxf(ax, bx), fmaxf(ay, by), fminf(fmaxf(az, bz), tmax));
  *tnear = tn;
  return tn <= tf;
}

// Both children of a binary node (vlbk::pack_node's layout) against a ray whose
// octant differs per lane: the same terms and min/max as slab_rt, the six
// pairs of plane crossings from six packed FMAs instead of twelve.
__device__ __forceinline__ void slab_pair_rt(const RayCtx& r, const float4 q0, const float4 q1, const float4 q2,
                                             float tmin, float tmax, bool& h0, bool& h1, float& tn0, float& tn1) {
  const float2 l0 = fma_pair(q0.x, q0.y, r.ixy, r.nxy), u0 = fma_pair(q0.z, q0.w, r.ixy, r.nxy);
  const float2 l1 = fma_pair(q1.x, q1.y, r.ixy, r.nxy), u1 = fma_pair(q1.z, q1.w, r.ixy, r.nxy);
  const float2 z0 = fma_pair(q2.x, q2.y, r.izz, r.nzz), z1 = fma_pair(q2.z, q2.w, r.izz, r.nzz);
  tn0 = fmax3(fminf(l0.x, u0.x), fminf(l0.y, u0.y), fmaxf(fminf(z0.x, z0.y), tmin));
  tn1 = fmax3(fminf(l1.x, u1.x), fminf(l1.y, u1.y), fmaxf(fminf(z1.x, z1.y), tmin));
  h0 = tn0 <= fmin3(fmaxf(l0.x, u0.x), fmaxf(l0.y, u0.y), fminf(fmaxf(z0.x, z0.y), tmax));
  h1 = tn1 <= fmin3(fmaxf(l1.x, u1.x), fmaxf(l1.y, u1.y), fminf(fmaxf(z1.x, z1.y), tmax));
}

__device__ __forceinline__ uint32_t lane_lt_mask() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// One lane's ray: its walk and the pending shading of its primary hit.
// cur: the next node (>= 0), triangle slot ~cur, or kWalkEnd; leaf: a
// triangle slot parked for the next leaf phase (-1 none).
constexpr int kWalkEnd = INT_MIN;
// First step of a walk: the root node, the one triangle of a one-triangle
// scene, or nothing in an empty scene.
__device__ __forceinline__ int walk_root(uint32_t ntris) { return ntris > 1 ? 0 : (ntris == 1 ? ~0 : kWalkEnd); }
struct LaneRay {
  bool has = false, shadow = false;
  uint32_t p = 0, s = 0;
  float ox = 0.f, oy = 0.f, oz = 0.f;
  float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
  RayCtx ray;
  int cur = 0, sp = 0, slot = -1, id = -1, leaf = -1;
  float tb = 0.f, lit = 0.f;
  // the lane's previous primary hit and shadow occluder (triangle slots or
  // -1): tested first by its next rays (see lr_start)
  int hprev = -1, oprev = -1;
};

// Warm start.  A lane's consecutive rays mostly share a probe and take
// neighbouring directions, so they often hit the same triangle, and shadow
// rays from nearby points toward the sun are often blocked by the same
// occluder.  Testing that triangle before the walk starts only tightens the
// best distance (or ends an occluded shadow walk at once): the closest hit is
// the minimum over all triangles with the same tie rule whatever order they
// are tested in, and an occluded shadow ray is occluded by any occluder, so
// every ray's result is unchanged.  A slot is tested only if it is a slot of
// the current scene (a lane of a batch may change scenes between rays).
template <class A>
__device__ __forceinline__ float lr_try(const A& a, const LaneRay& L, int ts, int* id) {
  ts = VLB_CLAMP(ts, a.ntris, a.err);
  const float4 v0 = __ldg(a.tris + 3 * ts), e1 = __ldg(a.tris + 3 * ts + 1), e2 = __ldg(a.tris + 3 * ts + 2);
  *id = __float_as_int(v0.w);
  return tri_hit(L.ray, v0, e1, e2);
}

// A: TraceArgs or BakeJobDev (scene, shading, probes and dirs fields).
template <class A>
__device__ __forceinline__ void lr_start(const A& a, LaneRay& L, uint32_t p, uint32_t s) {
  p = VLB_CLAMP(p, a.nprobes, a.err);
  s = VLB_CLAMP(s, a.S, a.err);
  L.p = p;
  L.s = s;
  L.d = __ldg(a.dirs + s);
  L.ox = a.probes[3 * size_t(p)];
  L.oy = a.probes[3 * size_t(p) + 1];
  L.oz = a.probes[3 * size_t(p) + 2];
  const float4 inv = __ldg(a.dinv + s);
  make_ray_inv(L.ray, L.ox, L.oy, L.oz, L.d.x, L.d.y, L.d.z, inv.x, inv.y, inv.z);
  L.has = true;
  L.shadow = false;
  L.cur = walk_root(a.ntris);
  L.sp = 0;
  L.slot = -1;
  L.id = -1;
  L.leaf = -1;
  L.tb = a.tmax;
  if (L.hprev >= 0 && uint32_t(L.hprev) < a.ntris) {
    int id;
    const float t = lr_try(a, L, L.hprev, &id);
    if (t > a.tmin && t < L.tb) { L.tb = t; L.slot = L.hprev; L.id = id; }
  }
}

// The reference baker's sample encoding: the sRGB curve of
// shaders/env_map.rchit:27-34 (the same in main.rmiss:9-16), then the 8-bit
// UNORM store of its R8G8B8A8 env map (round to nearest, clamped to [0, 1]).
__device__ __forceinline__ float ref_srgb(float c) {
  return c < 0.0031308f ? c * 12.92f : 1.055f * powf(c, 1.0f / 2.4f) - 0.055f;
}
__device__ __forceinline__ float ref_unorm8(float c) { return rintf(fminf(fmaxf(c, 0.f), 1.f) * 255.f) / 255.f; }

// The reference's shading of a primary result (vlb_shading
// VLB_SHADE_REF_PHONG, shaders/env_map.rchit:51-102): a miss is done; a hit
// facing the point light starts its shadow walk toward it (returns false;
// diffuse + specular wait in lit), any other hit is black.
template <class A>
__device__ __forceinline__ bool lr_finish_ref_primary(const A& a, LaneRay& L, Shaded& o) {
  if (L.slot < 0) {
    if (a.sky) {
      const float* tx =
          a.sky + 3 * size_t(VLB_CLAMP(cube_texel(L.d.x, L.d.y, L.d.z, a.sky_n), 6u * a.sky_n * a.sky_n, a.err));
      o.r = ref_unorm8(ref_srgb(__ldg(tx)));
      o.g = ref_unorm8(ref_srgb(__ldg(tx + 1)));
      o.b = ref_unorm8(ref_srgb(__ldg(tx + 2)));
    }
    return true;
  }
  L.slot = VLB_CLAMP(L.slot, a.ntris, a.err);
  const float4 e1 = __ldg(a.tris + 3 * L.slot + 1), e2 = __ldg(a.tris + 3 * L.slot + 2);
  o.tri = L.id;
  float nx = e1.y * e2.z - e1.z * e2.y, ny = e1.z * e2.x - e1.x * e2.z, nz = e1.x * e2.y - e1.y * e2.x;
  const float rn = rsqrtf(nx * nx + ny * ny + nz * nz);
  nx *= rn; ny *= rn; nz *= rn;
  const float px = fmaf(L.tb, L.d.x, L.ox), py = fmaf(L.tb, L.d.y, L.oy), pz = fmaf(L.tb, L.d.z, L.oz);
  const float sx = a.light.x - px, sy = a.light.y - py, sz = a.light.z - pz;
  const float len = sqrtf(sx * sx + sy * sy + sz * sz);
  const float lx = sx / len, ly = sy / len, lz = sz / len;
  const float sdn = fmaxf(lx * nx + ly * ny + lz * nz, 0.f);
  if (!(sdn > 0.f)) return true;  // no shadow ray: the sample stays black
  const float rdot = 2.f * (nx * lx + ny * ly + nz * lz);
  const float rx = lx - rdot * nx, ry = ly - rdot * ny, rz = lz - rdot * nz;
  float sp = fmaxf(rx * L.d.x + ry * L.d.y + rz * L.d.z, 0.f);
  sp *= sp; sp *= sp; sp *= sp; sp *= sp;  // ^16
  L.lit = 0.5f * sdn + 0.5f * sp;
  make_ray(L.ray, px + a.bias * nx, py + a.bias * ny, pz + a.bias * nz, lx, ly, lz);
  L.shadow = true;
  L.cur = walk_root(a.ntris);
  L.sp = 0;
  L.slot = -1;
  L.tb = len;
  if (L.oprev >= 0 && uint32_t(L.oprev) < a.ntris) {
    int id;
    const float t = lr_try(a, L, L.oprev, &id);
    if (t > 0.0f && t < L.tb) { L.slot = L.oprev; L.cur = kWalkEnd; }
  }
  return false;
}

// After a walk (REF: the reference's shading, vlb_shading
// VLB_SHADE_REF_PHONG; the kernels are built for one shading or the other).
// A finished primary walk is shaded: a miss takes the sky, a
// lit-facing hit starts its shadow walk (returns false: the lane walks on,
// the triangle id and sun term wait in id / lit), anything else is done.  A
// finished shadow walk gives the Lambert term or 0.  Returns true with the
// sample in `o` when the ray is complete.
template <bool COUNT, class A, bool REF = false>
__device__ __forceinline__ bool lr_finish(const A& a, LaneRay& L, Shaded& o, Work& w) {
  o = Shaded{0.f, 0.f, 0.f, -1, 2};
  if constexpr (REF) {
    if (!L.shadow) {
      L.hprev = L.slot;
      return lr_finish_ref_primary(a, L, o);
    }
  }
  if (!L.shadow) {
    L.hprev = L.slot;
    if (L.slot < 0) {
      if (a.sky) {
        const float* tx =
            a.sky + 3 * size_t(VLB_CLAMP(cube_texel(L.d.x, L.d.y, L.d.z, a.sky_n), 6u * a.sky_n * a.sky_n, a.err));
        o.r = __ldg(tx); o.g = __ldg(tx + 1); o.b = __ldg(tx + 2);
      }
      return true;
    }
    L.slot = VLB_CLAMP(L.slot, a.ntris, a.err);
    const float4 e1 = __ldg(a.tris + 3 * L.slot + 1), e2 = __ldg(a.tris + 3 * L.slot + 2);
    o.tri = L.id;
    float nx = e1.y * e2.z - e1.z * e2.y, ny = e1.z * e2.x - e1.x * e2.z, nz = e1.x * e2.y - e1.y * e2.x;
    const float rn = rsqrtf(nx * nx + ny * ny + nz * nz);
    nx *= rn; ny *= rn; nz *= rn;
    if (nx * L.d.x + ny * L.d.y + nz * L.d.z > 0.f) { nx = -nx; ny = -ny; nz = -nz; }
    const float ndl = nx * a.sun.x + ny * a.sun.y + nz * a.sun.z;
    if (!(ndl > 0.f)) return true;
    if constexpr (COUNT) ++w.shadow;
    make_ray_inv(L.ray, fmaf(L.tb, L.d.x, L.ox) + a.bias * nx, fmaf(L.tb, L.d.y, L.oy) + a.bias * ny,
                 fmaf(L.tb, L.d.z, L.oz) + a.bias * nz, a.sun.x, a.sun.y, a.sun.z, a.sun_inv.x, a.sun_inv.y,
                 a.sun_inv.z);
    L.lit = a.sun_scale * ndl;
    L.shadow = true;
    L.cur = walk_root(a.ntris);
    L.sp = 0;
    L.slot = -1;
    L.tb = a.tmax;
    if (L.oprev >= 0 && uint32_t(L.oprev) < a.ntris) {
      int id;
      const float t = lr_try(a, L, L.oprev, &id);
      if (t > 0.0f && t < L.tb) { L.slot = L.oprev; L.cur = kWalkEnd; }
    }
    return false;
  }
  o.tri = L.id;
  const bool occ = L.slot >= 0;
  if (occ) L.oprev = L.slot;
  o.vis = occ ? 0 : 1;
  if (!occ) {
    const float4 alb = __ldg(a.albedo + VLB_CLAMP(L.id, a.ntris, a.err));
    if constexpr (REF) {
      o.r = ref_unorm8(ref_srgb(alb.x * L.lit));
      o.g = ref_unorm8(ref_srgb(alb.y * L.lit));
      o.b = ref_unorm8(ref_srgb(alb.z * L.lit));
    } else {
      o.r = alb.x * L.lit; o.g = alb.y * L.lit; o.b = alb.z * L.lit;
    }
  }
  return true;
}

// Speculative while-while walk.  Run one step per turn, a warp's lanes at an
// inner node and its lanes at a (single-triangle) leaf take different
// branches nearly every turn.  Here a turn has a node phase -- every lane
// walks inner nodes until it meets a leaf, parks it (one slot), and walks on
// past it while other lanes of the warp still look for theirs -- and then a
// leaf phase in which all parked triangles are tested together.  Only the
// visiting order changes: box tests are conservative, pruning keeps a margin
// and ties go to the lower triangle id, so every ray's result is unchanged.
__device__ __forceinline__ bool lr_is_tri(int cur) { return cur < 0 && cur != kWalkEnd; }

__device__ __forceinline__ void lr_park(LaneRay& L, const int* stack) {
  if (L.has && L.leaf < 0 && lr_is_tri(L.cur)) {
    L.leaf = ~L.cur;
    L.cur = L.sp ? stack[--L.sp] : kWalkEnd;
  }
}

// Byte c (0..3) of a word as an exact float.
__device__ __forceinline__ float q8(uint32_t word, int c) {
  return __uint_as_float(0x4B000000u | ((word >> (8 * c)) & 255u)) - 8388608.0f;
}

// One node of the 8-wide quantised tree (layout in wide_bvh.cpp): every valid
// child's box is dequantised with the build's FP32 expression fmaf(q, 2^e,
// origin) -- a box that contains the binary tree's box for that subtree --
// and slab-tested as in the binary walk; the nearest hit child is next, the
// other hit children go on the stack.  The children are tested four at a
// time (their bound bytes are six words) and a child's reference is read only
// when its box is hit, to keep the walk's registers few.
template <bool COUNT, class A>
__device__ __forceinline__ void lr_node_wide(const A& a, LaneRay& L, int* stack, Work& w) {
  if (!VLB_INB(L.cur, a.nwide, a.err)) { L.cur = kWalkEnd; L.sp = 0; return; }
  if constexpr (COUNT) { ++w.wnodes; ++w.lnodes; }
  const float tlo = L.shadow ? 0.0f : a.tmin;
  const float4* nd = a.wnodes + 6 * size_t(L.cur);
  const float4 h = __ldg(nd);
  const int* refs = reinterpret_cast<const int*>(nd + 4);
  const uint32_t meta = __float_as_uint(h.w);
  const float sx = __uint_as_float((meta & 255u) << 23), sy = __uint_as_float(((meta >> 8) & 255u) << 23),
              sz = __uint_as_float(((meta >> 16) & 255u) << 23);
  const int nc = int(meta >> 24);
  const float lim = prune_limit(L.tb);
  int next = kWalkEnd;
  float tnext = INFINITY;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    if (4 * half >= nc) break;
    uint32_t q[6];  // lo x, hi x, lo y, hi y, lo z, hi z: one byte per child
    if (half == 0) {
      const uint4 u = __ldg(reinterpret_cast<const uint4*>(nd + 1));
      const uint2 v = __ldg(reinterpret_cast<const uint2*>(nd + 2));
      q[0] = u.x; q[1] = u.y; q[2] = u.z; q[3] = u.w; q[4] = v.x; q[5] = v.y;
    } else {
      const uint2 v = __ldg(reinterpret_cast<const uint2*>(nd + 2) + 1);
      const uint4 u = __ldg(reinterpret_cast<const uint4*>(nd + 3));
      q[0] = v.x; q[1] = v.y; q[2] = u.x; q[3] = u.y; q[4] = u.z; q[5] = u.w;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (4 * half + c < nc) {
        const float lx = fmaf(q8(q[0], c), sx, h.x), hx = fmaf(q8(q[1], c), sx, h.x);
        const float ly = fmaf(q8(q[2], c), sy, h.y), hy = fmaf(q8(q[3], c), sy, h.y);
        const float lz = fmaf(q8(q[4], c), sz, h.z), hz = fmaf(q8(q[5], c), sz, h.z);
        float tn;
        if (slab_rt(L.ray, lx, ly, lz, hx, hy, hz, tlo, lim, &tn)) {
          const int ref = __ldg(refs + 4 * half + c);
          int push = ref;
          if (tn < tnext) {
            push = next;
            next = ref;
            tnext = tn;
          }
          if (push != kWalkEnd) {
            if (L.sp < kLaneStack) stack[L.sp++] = push;
            else atomicAdd(a.err + kErrStackOverflow, 1);
          }
        }
      }
    }
  }
  L.cur = next != kWalkEnd ? next : (L.sp ? stack[--L.sp] : kWalkEnd);
}

// slab_pair_rt for a ray in octant OCT (bit a set: 1/d_a < 0): each axis's
// entry and exit planes are known, so the per-axis min/max goes.  The same
// bits as slab_pair_rt: a plane crossing fma(p, inv, -o * inv) is monotone in
// p, so the entry plane's crossing is the minimum of the two.  (A crossing is
// NaN only when p * inv and o * inv both overflow -- a direction component
// below 1e-30, so inv = +-1e30, with coordinates beyond 3.4e8 -- and there
// the two forms may differ, as the packet walk's compile-time octant may.)
template <int OCT>
__device__ __forceinline__ void slab_pair_oct(const RayCtx& r, const float4 q0, const float4 q1, const float4 q2,
                                              float tmin, float tmax, bool& h0, bool& h1, float& tn0, float& tn1) {
  constexpr bool fx = OCT & 1, fy = OCT & 2, fz = OCT & 4;
  const float2 l0 = fma_pair(q0.x, q0.y, r.ixy, r.nxy), u0 = fma_pair(q0.z, q0.w, r.ixy, r.nxy);
  const float2 l1 = fma_pair(q1.x, q1.y, r.ixy, r.nxy), u1 = fma_pair(q1.z, q1.w, r.ixy, r.nxy);
  const float2 z0 = fma_pair(q2.x, q2.y, r.izz, r.nzz), z1 = fma_pair(q2.z, q2.w, r.izz, r.nzz);
  tn0 = fmax3(fx ? u0.x : l0.x, fy ? u0.y : l0.y, fmaxf(fz ? z0.y : z0.x, tmin));
  tn1 = fmax3(fx ? u1.x : l1.x, fy ? u1.y : l1.y, fmaxf(fz ? z1.y : z1.x, tmin));
  h0 = tn0 <= fmin3(fx ? l0.x : u0.x, fy ? l0.y : u0.y, fminf(fz ? z0.x : z0.y, tmax));
  h1 = tn1 <= fmin3(fx ? l1.x : u1.x, fy ? l1.y : u1.y, fminf(fz ? z1.x : z1.y, tmax));
}

// The octant every lane with a ray shares (-1 if they differ).  A lane's ray
// changes only between node phases, so one vote serves a whole phase.
__device__ __forceinline__ int lr_warp_octant(const LaneRay& L) {
  const int o = (L.ray.ixy.x < 0.f ? 1 : 0) | (L.ray.ixy.y < 0.f ? 2 : 0) | (L.ray.izz.x < 0.f ? 4 : 0);
  const unsigned has = __ballot_sync(kFull, L.has);
  if (!has) return -1;
  const int first = __shfl_sync(kFull, o, __ffs(has) - 1);
  return __all_sync(kFull, !L.has || o == first) ? first : -1;
}

// One inner node: nearer hit child next, the farther one on the stack.  WIDE:
// the node is a node of the 8-wide tree (kernels built for it walk it when
// the scene has one; the others walk the binary tree, with the same results).
// PACKED: the box tests' plane crossings by packed FMAs (slab_pair_rt), else
// by scalar ones (slab_rt; the same bits, for kernels whose registers do not
// leave room for the pairs).  OCT >= 0: the lane's ray is in that octant
// (slab_pair_oct).
template <bool COUNT, class A, bool WIDE = false, bool PACKED = true, int OCT = -1>
__device__ __forceinline__ void lr_node(const A& a, LaneRay& L, int* stack, Work& w) {
  if constexpr (WIDE) {
    lr_node_wide<COUNT>(a, L, stack, w);
    return;
  }
  if (!VLB_INB(L.cur, 2 * a.ntris - 2, a.err)) { L.cur = kWalkEnd; L.sp = 0; return; }
  if constexpr (COUNT) { ++w.wnodes; ++w.lnodes; }
  const float tlo = L.shadow ? 0.0f : a.tmin;
  float4 n0, n1, n2, n3;
  ldg_node(a.nodes + 4 * L.cur, n0, n1, n2, n3);
  float tn0, tn1;
  bool h0, h1;
  if constexpr (OCT >= 0) {
    slab_pair_oct<OCT>(L.ray, n0, n1, n2, tlo, prune_limit(L.tb), h0, h1, tn0, tn1);
  } else if constexpr (PACKED) {
    slab_pair_rt(L.ray, n0, n1, n2, tlo, prune_limit(L.tb), h0, h1, tn0, tn1);
  } else {
    const float lim = prune_limit(L.tb);
    h0 = slab_rt(L.ray, n0.x, n0.y, n2.x, n0.z, n0.w, n2.y, tlo, lim, &tn0);
    h1 = slab_rt(L.ray, n1.x, n1.y, n2.z, n1.z, n1.w, n2.w, tlo, lim, &tn1);
  }
  const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
  if (h0 && h1) {
    const bool first0 = tn0 <= tn1;
    if (L.sp < kLaneStack) stack[L.sp++] = first0 ? c1 : c0;
    else atomicAdd(a.err + kErrStackOverflow, 1);
    L.cur = first0 ? c0 : c1;
  } else if (h0) {
    L.cur = c0;
  } else if (h1) {
    L.cur = c1;
  } else {
    L.cur = L.sp ? stack[--L.sp] : kWalkEnd;
  }
}

// The parked triangle; an occluder ends a shadow walk.
template <bool COUNT, class A>
__device__ __forceinline__ void lr_leaf(const A& a, LaneRay& L, Work& w) {
  if constexpr (COUNT) ++w.wtris;
  const int ts = VLB_CLAMP(L.leaf, a.ntris, a.err);
  L.leaf = -1;
  const float tlo = L.shadow ? 0.0f : a.tmin;
  const float4 v0 = __ldg(a.tris + 3 * ts), e1 = __ldg(a.tris + 3 * ts + 1), e2 = __ldg(a.tris + 3 * ts + 2);
  const float t = tri_hit(L.ray, v0, e1, e2);
  if (!(t > tlo)) return;
  if (L.shadow) {
    if (t < L.tb) { L.slot = ts; L.cur = kWalkEnd; L.sp = 0; }
    return;
  }
  const int tid = __float_as_int(v0.w);
  if (t < L.tb || (t == L.tb && L.slot >= 0 && tid < L.id)) { L.tb = t; L.slot = ts; L.id = tid; }
}

// Up to `steps` node steps of the warp's lanes (every lane takes part in the
// votes); OCT: the octant all the warp's rays share, or -1.
template <bool COUNT, class A, bool WIDE, bool PACKED, int OCT>
__device__ __forceinline__ void lr_node_steps(const A& a, LaneRay& L, int* stack, Work& w, uint32_t steps) {
#pragma unroll 1
  for (uint32_t k = 0; k < steps; ++k) {
    lr_park(L, stack);
    const bool at_node = L.has && L.cur >= 0;
    if (!__any_sync(kFull, at_node && L.leaf < 0)) break;
    if (at_node) lr_node<COUNT, A, WIDE, PACKED, OCT>(a, L, stack, w);
  }
}

// A turn's node phase, specialised to the warp's octant when all its rays
// share one (the binary tree's packed walk; the others take the generic one).
// Measured on the single-bake tile walk: 129.3 -> 125.7 ms on the bake of
// 64^3 probes x 1024 directions in the 4096-box scene; the multi-job walks
// measured 4 % slower with it (also when only jobs of 1024 directions took
// it) and keep the generic phase.
template <bool COUNT, class A, bool WIDE = false, bool PACKED = true>
__device__ __forceinline__ void lr_node_phase(const A& a, LaneRay& L, int* stack, Work& w, uint32_t steps) {
  if constexpr (WIDE || !PACKED) {
    lr_node_steps<COUNT, A, WIDE, PACKED, -1>(a, L, stack, w, steps);
  } else {
    switch (lr_warp_octant(L)) {
      case 0: lr_node_steps<COUNT, A, false, true, 0>(a, L, stack, w, steps); break;
      case 1: lr_node_steps<COUNT, A, false, true, 1>(a, L, stack, w, steps); break;
      case 2: lr_node_steps<COUNT, A, false, true, 2>(a, L, stack, w, steps); break;
      case 3: lr_node_steps<COUNT, A, false, true, 3>(a, L, stack, w, steps); break;
      case 4: lr_node_steps<COUNT, A, false, true, 4>(a, L, stack, w, steps); break;
      case 5: lr_node_steps<COUNT, A, false, true, 5>(a, L, stack, w, steps); break;
      case 6: lr_node_steps<COUNT, A, false, true, 6>(a, L, stack, w, steps); break;
      case 7: lr_node_steps<COUNT, A, false, true, 7>(a, L, stack, w, steps); break;
      default: lr_node_steps<COUNT, A, false, true, -1>(a, L, stack, w, steps); break;
    }
  }
}

constexpr int kNodeSteps = 6;   // bound on one turn's node phase
constexpr int kRefillIdle = 32; // idle lanes that trigger a refill: a whole idle warp (measured fastest)

}  // namespace vlbk
