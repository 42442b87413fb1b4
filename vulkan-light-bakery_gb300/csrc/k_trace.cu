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
// ballots decide which children to visit.  All control flow is warp-uniform.
// The stack is warp-uniform too, so it lives in registers spread over the
// lanes (entry i in lane i % 32) and a pop is one shuffle.  A lane tests only
// the nodes its own box tests admit (one private bit per stack entry), and
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
// Lane mode.  When a packet's probes are far apart relative to the
// geometry (few probes in a large scene) the union of their paths is much
// longer than any one path, so each lane walks its own path instead (a
// per-lane stack in local memory, the warp's direction -- and octant -- still
// shared).  Both modes prune a subtree only when its box entry exceeds the
// lane's best distance by a relative margin of 2^-12, so a triangle whose
// computed distance ties or beats the best is never pruned by a rounding of
// the box test: a lane's result does not depend on the visiting order, hence
// on the mode or the packet.
//
// Scheduling: persistent, independent warps take work items (packet,
// direction chunk) from an atomic counter -- no CTA-wide barrier, so a warp
// that drew cheap directions moves on at once.  Fused mode accumulates each
// probe's K x 3 coefficients over the chunk in shared memory
// (lane-contiguous), writes one partial per item, and the last item of a
// packet (atomic ticket) adds the partials in FP64 in chunk order.  Every
// probe's sums therefore have the same order whatever the batch and the
// scheduling.  Tile mode writes the [probe][3][S] radiance tile instead (the
// plain path).
#include <cuda_bf16.h>

#include <algorithm>
#include <climits>

#include "trace_common.cuh"
#include "vlb_device.cuh"
#include "vlb_internal.h"

namespace vlbk {

// MODE 0: radiance tile (+ optional per-ray debug arrays); MODE 1: fused projection.
// Every warp is persistent and independent: lane 0 takes the next work item
// (packet, direction chunk) from the counter; no CTA-wide barrier anywhere.
template <int MODE, int K, bool COUNT>
__global__ void __launch_bounds__(kTraceThreads) k_trace(const TraceArgs a) {
  constexpr int V = 3 * K;
  constexpr int AW = MODE == 1 ? kTraceWarps : 1, AV = MODE == 1 ? V : 1;
  __shared__ float acc[AW][AV][32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t npg = (a.nprobes + 31) / 32;
  const uint32_t total = npg * a.chunks;
  Work w;
  for (;;) {
    uint32_t item = 0;
    if (lane == 0) item = atomicAdd(a.work_counter, 1u);
    item = __shfl_sync(kFull, item, 0);
    if (item >= total) break;
    // chunk-major: the warps in flight trace neighbouring chunks of the
    // octant-grouped direction order, i.e. mostly one traversal variant
    const uint32_t chunk = item / npg, pg = item - chunk * npg;
    const uint32_t slot = pg * 32 + lane;
    const bool valid = slot < a.nprobes;
    const uint32_t p = valid ? VLB_CLAMP(a.order[slot], a.nprobes, a.err) : 0;
    const float ox = valid ? a.probes[3 * size_t(p)] : 0.f, oy = valid ? a.probes[3 * size_t(p) + 1] : 0.f,
                oz = valid ? a.probes[3 * size_t(p) + 2] : 0.f;
    const uint32_t s0 = min(a.S, chunk * a.dirs_per_warp), s1 = min(a.S, s0 + a.dirs_per_warp);
    if constexpr (MODE == 1) {
#pragma unroll
      for (int v = 0; v < V; ++v) acc[warp][v][lane] = 0.f;
    }
    for (uint32_t t = s0; t < s1; ++t) {
      const uint32_t s = VLB_CLAMP(__ldg(a.dir_order + t), a.S, a.err);  // direction index (caller order)
      const float4 dv = __ldg(a.dirs + s);
      const Shaded o = a.lane ? trace_sample<COUNT, true>(a, valid, ox, oy, oz, dv, w)
                              : trace_sample<COUNT, false>(a, valid, ox, oy, oz, dv, w);
      if constexpr (MODE == 1) {
        const float4* b4 = reinterpret_cast<const float4*>(a.basis16 + size_t(s) * 16);
#pragma unroll
        for (int q = 0; q < (K + 3) / 4; ++q) {
          const float4 b = __ldg(b4 + q);
          const float bb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int k = 4 * q + e;
            if (k < K) {
              acc[warp][3 * k][lane] = fmaf(bb[e], o.r, acc[warp][3 * k][lane]);
              acc[warp][3 * k + 1][lane] = fmaf(bb[e], o.g, acc[warp][3 * k + 1][lane]);
              acc[warp][3 * k + 2][lane] = fmaf(bb[e], o.b, acc[warp][3 * k + 2][lane]);
            }
          }
        }
      }
      if (!valid) continue;
      const size_t ri = size_t(p) * a.S + s;
      if (a.hit_tri) a.hit_tri[ri] = o.tri;
      if (a.shadow) a.shadow[ri] = o.vis;
      if constexpr (MODE == 0) {
        const size_t row = size_t(p) * 3;
        if (a.radiance) {
          a.radiance[row * a.S + s] = o.r;
          a.radiance[(row + 1) * a.S + s] = o.g;
          a.radiance[(row + 2) * a.S + s] = o.b;
        }
        if (a.radiance_bf16) {
          store_bf16(a.radiance_bf16, row, a.S, s, o.r, a.bf16_split);
          store_bf16(a.radiance_bf16, row + 1, a.S, s, o.g, a.bf16_split);
          store_bf16(a.radiance_bf16, row + 2, a.S, s, o.b, a.bf16_split);
        }
        if (a.dbg_radiance) {
          a.dbg_radiance[3 * ri] = o.r; a.dbg_radiance[3 * ri + 1] = o.g; a.dbg_radiance[3 * ri + 2] = o.b;
        }
      }
    }
    if constexpr (MODE == 1) {
      __syncwarp();
      if (a.chunks == 1) {
        if (valid)
          for (int v = 0; v < V; ++v) a.out[size_t(p) * V + v] = acc[warp][v][lane];
        continue;
      }
      if (valid)
        for (int v = 0; v < V; ++v) a.partial[(size_t(p) * a.chunks + chunk) * V + v] = acc[warp][v][lane];
      // the last item of this packet adds the chunk partials in FP64, in chunk order
      __threadfence();
      __syncwarp();
      uint32_t ticket = 0;
      if (lane == 0) ticket = atomicAdd(a.group_done + pg, 1u);
      ticket = __shfl_sync(kFull, ticket, 0);
      if (ticket == a.chunks - 1) {
        __threadfence();
        if (valid) {
          const float* src = a.partial + size_t(p) * a.chunks * V;
          for (int v = 0; v < V; ++v) {
            double s = 0.0;
            for (uint32_t j = 0; j < a.chunks; ++j) s += double(__ldcg(src + size_t(j) * V + v));
            a.out[size_t(p) * V + v] = float(s);
          }
        }
      }
    }
  }
  if constexpr (COUNT) {
    atomicAdd(a.counters + 0, (unsigned long long)w.wnodes);
    atomicAdd(a.counters + 1, (unsigned long long)w.wtris);
    atomicAdd(a.counters + 2, (unsigned long long)w.shadow);
    atomicAdd(a.counters + 3, (unsigned long long)w.lnodes);
  }
}

void plan_trace(TraceArgs& a, int num_sms, bool fused) {
  const uint64_t npg = (uint64_t(a.nprobes) + 31) / 32;
  // items: ~8 per resident warp for balance (tile mode); in fused mode each
  // extra chunk costs a K x 3 partial per probe, so stop at ~2 per warp
  const uint64_t warps = uint64_t(num_sms) * 32;
  const uint64_t target = fused ? 2 * warps : 8 * warps;
  uint64_t chunks = (target + npg - 1) / npg;
  chunks = std::max<uint64_t>(1, std::min<uint64_t>(chunks, a.S ? a.S : 1));
  const uint64_t dpw = std::max<uint64_t>(1, (uint64_t(a.S) + chunks - 1) / chunks);
  a.dirs_per_warp = uint32_t(dpw);
  a.chunks = uint32_t(std::max<uint64_t>(1, (uint64_t(a.S) + dpw - 1) / dpw));
}

template <int MODE, int K, bool COUNT>
static void launch(const TraceArgs& a, int num_sms, cudaStream_t s) {
  const uint64_t items = ((uint64_t(a.nprobes) + 31) / 32) * a.chunks;
  if (!items) return;
  static int per_sm = 0;  // resident CTAs per SM for this instantiation
  if (!per_sm) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace<MODE, K, COUNT>, kTraceThreads, 0);
    if (per_sm < 1) per_sm = 1;
  }
  const uint64_t ctas = std::min<uint64_t>((items + kTraceWarps - 1) / kTraceWarps, uint64_t(num_sms) * per_sm);
  k_trace<MODE, K, COUNT><<<uint32_t(ctas), kTraceThreads, 0, s>>>(a);
}

// ---- lane mode with per-lane ray fetch (tile output) ---------------------------------
// Persistent warps; every lane runs its own ray through a small state machine
// -- primary walk, shading, shadow walk, output -- and takes a new ray as
// soon as it is done (a turn walks nodes until the warp's lanes have each
// found a leaf, then tests those leaves: lr_node / lr_leaf).  Idle lanes refill
// together from a global ray counter (one atomic per refill, when half the
// warp or all of it is idle), so a warp no longer waits for its slowest ray
// and primary and shadow walks of different rays overlap.  Ray r is
// (probe slot r / S, direction position r % S): rays fetched together share
// their origin and take neighbouring directions of the trace order (grouped
// by octant, then by position on the octant's face), so their walks share
// the nodes around the probe (5 % faster than rays of one direction from
// Morton-neighbour probes on a 16^3 grid, 19 % on random probes); slots run
// to the probe count rounded up to 32.  Box tests take the per-lane octant
// at run time; the tests, the pruning and the tie rule are those of
// lane_traverse, so each ray's result is unchanged.

// A finished ray's tile entries (and debug arrays).
__device__ __forceinline__ void emit_tile(const TraceArgs& a, const LaneRay& L, const Shaded& o) {
  if (!VLB_INB(L.p, a.nprobes, a.err) || !VLB_INB(L.s, a.S, a.err)) return;
  const size_t ri = size_t(L.p) * a.S + L.s, row = size_t(L.p) * 3;
  if (a.hit_tri) a.hit_tri[ri] = o.tri;
  if (a.shadow) a.shadow[ri] = o.vis;
  if (a.radiance) {
    a.radiance[row * a.S + L.s] = o.r;
    a.radiance[(row + 1) * a.S + L.s] = o.g;
    a.radiance[(row + 2) * a.S + L.s] = o.b;
  }
  if (a.radiance_bf16) {
    store_bf16(a.radiance_bf16, row, a.S, L.s, o.r, a.bf16_split);
    store_bf16(a.radiance_bf16, row + 1, a.S, L.s, o.g, a.bf16_split);
    store_bf16(a.radiance_bf16, row + 2, a.S, L.s, o.b, a.bf16_split);
  }
  if (a.dbg_radiance) {
    a.dbg_radiance[3 * ri] = o.r; a.dbg_radiance[3 * ri + 1] = o.g; a.dbg_radiance[3 * ri + 2] = o.b;
  }
}

template <bool COUNT, bool WIDE, bool REF>
// Nine resident CTAs per SM (at most 56 registers): measured 4 % faster on
// the 64^3-probe, 1024-direction bake than the unconstrained 60 registers
// (eight CTAs: 130.9 against 125.6 ms); ten CTAs would spill.
__global__ void __launch_bounds__(kTraceThreads, 9) k_trace_dyn(const TraceArgs a) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t P = (a.nprobes + 31) / 32 * 32;
  const uint32_t R = P * a.S;
  Work w;
  int stack[kLaneStack];
  LaneRay L;
  make_ray(L.ray, 0.f, 0.f, 0.f, 1.f, 1.f, 1.f);
  bool exhausted = false;
  // A warp takes its rays in blocks of `block` consecutive rays (whole 32-ray
  // groups of one probe's neighbouring directions) and hands a block's groups
  // to its lanes one by one: its next rays then reuse the nodes its last ones
  // fetched.  Blocks are sized by the rays per warp, so that every warp still
  // takes about 64 blocks (the load stays balanced): up to 16 groups on the
  // 64^3-probe, 1024-direction bake (9.5 % faster than one group), one group
  // on small bakes.
  // the warp's block (next ray, end) lives in shared memory: it is touched only
  // when the warp takes rays, and the walk's registers stay free
  __shared__ uint32_t s_block[kTraceWarps][2];
  uint32_t* wblk = s_block[threadIdx.x >> 5];
  if (lane == 0) { wblk[0] = 0; wblk[1] = 0; }
  __syncwarp();
  for (;;) {
    const unsigned idle = __ballot_sync(kFull, !L.has);
    if (!exhausted && idle == kFull) {  // a whole idle warp takes its next 32 rays together
      const uint32_t block = a.ray_block;  // set by the launch: the kernel's registers stay free
      uint32_t wb;
      if (block == 32) {  // one group a block: straight from the counter
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(a.work_counter, 32u);
        wb = __shfl_sync(kFull, base, 0);
        if (wb >= R) exhausted = true;
      } else {
        wb = wblk[0];
        if (wb >= wblk[1]) {
          uint32_t base = 0;
          if (lane == 0) base = atomicAdd(a.work_counter, block);
          base = __shfl_sync(kFull, base, 0);
          wb = base;
          if (base >= R) exhausted = true;
          __syncwarp();
          if (lane == 0) wblk[1] = base + block;
        }
        __syncwarp();
        if (lane == 0) wblk[0] = wb + 32;
        __syncwarp();
      }
      const uint32_t r = wb + lane;
      if (r < R) {
        const uint32_t sl = r / a.S, t = r - sl * a.S;
        if (sl < a.nprobes) lr_start(a, L, a.order[sl], __ldg(a.dir_order + t));
      }
    }
    if (!__any_sync(kFull, L.has)) {
      if (exhausted) break;
      continue;
    }
    // node phase (all lanes take part in the votes)
    lr_node_phase<COUNT, TraceArgs, WIDE>(a, L, stack, w, kNodeSteps);
    lr_park(L, stack);
    if (!L.has) continue;
    // leaf phase
    if (L.leaf >= 0) lr_leaf<COUNT>(a, L, w);
    if (L.cur != kWalkEnd) continue;
    Shaded o;
    if (!lr_finish<COUNT, TraceArgs, REF>(a, L, o, w)) continue;
    L.has = false;
    emit_tile(a, L, o);
  }
  if constexpr (COUNT) {
    atomicAdd(a.counters + 0, (unsigned long long)w.wnodes);
    atomicAdd(a.counters + 1, (unsigned long long)w.wtris);
    atomicAdd(a.counters + 2, (unsigned long long)w.shadow);
    atomicAdd(a.counters + 3, (unsigned long long)w.lnodes);
  }
}

template <bool COUNT, bool WIDE, bool REF>
static void launch_dyn(const TraceArgs& a, int num_sms, cudaStream_t s) {
  auto kern = k_trace_dyn<COUNT, WIDE, REF>;
  static int per_sm = 0;
  if (!per_sm) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTraceThreads, 0);
    if (per_sm < 1) per_sm = 1;
  }
  const uint64_t rays = uint64_t((a.nprobes + 31) / 32 * 32) * a.S;
  const uint64_t ctas = std::max<uint64_t>(
      std::min<uint64_t>((rays + kTraceThreads - 1) / kTraceThreads, uint64_t(num_sms) * per_sm), 1);
  // ray blocks: whole 32-ray groups, as many as keep ~64 blocks a warp, at most 16
  TraceArgs b = a;
  const uint64_t groups_per_warp = (rays / 32) / (ctas * kTraceWarps);
  b.ray_block = 32u * uint32_t(std::min<uint64_t>(16, std::max<uint64_t>(1, groups_per_warp / 64)));
  kern<<<uint32_t(ctas), kTraceThreads, 0, s>>>(b);
}

// The ray counter runs past R by at most one ray block (512) per resident warp: R < 2^31 keeps it in 32 bits.
bool trace_dyn_supported(const TraceArgs& a) {
  return a.lane && a.ntris > 0 && a.ntris < 0x7fffffffu &&
         uint64_t((a.nprobes + 31) / 32 * 32) * a.S < (1ull << 31);
}

// ---- grid mode: parallel rays through per-direction triangle grids -----------------
// Every probe of a bake traces the same directions and every shadow ray goes
// toward the sun, so the rays of one direction are parallel.  For each
// direction (grid g < S) and for the sun (grid S) one CTA projects the
// triangles onto a plane across the direction, bins their 2D boxes (widened
// by a margin) into a G x G grid over the projected scene and sorts each
// cell by near depth.  A ray then visits only the cell of its 2D point:
// entries that end before its interval are skipped, entries whose widened
// box misses the point are skipped, and the rest are tested with tri_hit in
// near-depth order until the next entry's nearest possible depth exceeds
// the pruning limit of the best hit (the tree walks' margin).  Every
// triangle tri_hit can report for the ray is in that cell (the margin,
// 2^-12 of the scene's coordinate scale, covers the FP32 projection error of
// triangles and of origins within grid_far of the origin), so each ray's
// result is that of the tree walks.  A grid whose entries overflow its
// capacity, and origins beyond grid_far, walk the tree instead.

// Monotone cell index (the same function bins the boxes and locates rays).
__device__ __forceinline__ uint32_t grid_cell(float x, float lo, float inv, uint32_t G) {
  return uint32_t(fminf(fmaxf((x - lo) * inv, 0.f), float(G - 1)));
}

// A basis (u, v) across d (any: exactness comes from the margins).
__device__ __forceinline__ void grid_basis(float dx, float dy, float dz, float3& u, float3& v) {
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  const float cx = (ax <= ay && ax <= az) ? 1.f : 0.f;
  const float cy = (cx == 0.f && ay <= az) ? 1.f : 0.f;
  const float cz = (cx == 0.f && cy == 0.f) ? 1.f : 0.f;
  float ux = dy * cz - dz * cy, uy = dz * cx - dx * cz, uz = dx * cy - dy * cx;
  const float rn = rsqrtf(ux * ux + uy * uy + uz * uz);
  ux *= rn; uy *= rn; uz *= rn;
  u = make_float3(ux, uy, uz);
  v = make_float3(dy * uz - dz * uy, dz * ux - dx * uz, dx * uy - dy * ux);
}

__device__ __forceinline__ float dot3(float x, float y, float z, float3 a) {
  return fmaf(z, a.z, fmaf(y, a.y, x * a.x));
}

size_t grid_build_smem(uint32_t G, uint32_t ntris) {
  return (2 * size_t(G) * G + 1) * 4 + size_t(ntris) * 8 + size_t(kGridCap) * 2;
}

// Block-wide exclusive scan of v[0, n) in place (kGridThreads threads, runs of
// ceil(n / threads) per thread); returns the total.
__device__ uint32_t grid_scan(uint32_t* v, uint32_t n, uint32_t* wsum) {
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t per = (n + kGridThreads - 1) / kGridThreads, c0 = tid * per;
  uint32_t run = 0;
  for (uint32_t k = 0; k < per; ++k)
    if (c0 + k < n) run += v[c0 + k];
  uint32_t inc = run;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, inc, o);
    if (int(lane) >= o) inc += y;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  uint32_t off = 0, total = 0;
  for (uint32_t k = 0; k < kGridThreads / 32; ++k) {
    if (k < warp) off += wsum[k];
    total += wsum[k];
  }
  off += inc - run;
  for (uint32_t k = 0; k < per; ++k)
    if (c0 + k < n) {
      const uint32_t x = v[c0 + k];
      v[c0 + k] = off;
      off += x;
    }
  __syncthreads();
  return total;
}

// One CTA per grid.  Shared memory: counts / start offsets (G*G+1), fill
// cursors (G*G), per triangle its packed cell range and near depth, then the
// entries.
__global__ void __launch_bounds__(kGridThreads) k_grid_build(const TraceArgs a) {
  extern __shared__ __align__(16) uint8_t gsm[];
  const uint32_t G = a.grid_g, GG = G * G, T = a.ntris;
  uint32_t* start = reinterpret_cast<uint32_t*>(gsm);
  uint32_t* cur = start + GG + 1;
  uint32_t* tcell = cur + GG;
  float* tnear = reinterpret_cast<float*>(tcell + T);
  uint16_t* ent = reinterpret_cast<uint16_t*>(tnear + T);
  __shared__ float red[4][kGridThreads / 32];
  __shared__ uint32_t wsum[kGridThreads / 32];
  const uint32_t gi = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float dx, dy, dz;
  if (gi < a.S) {
    const float4 d = __ldg(a.dirs + gi);
    dx = d.x; dy = d.y; dz = d.z;
  } else {
    dx = a.sun.x; dy = a.sun.y; dz = a.sun.z;
  }
  float3 u, v;
  grid_basis(dx, dy, dz, u, v);
  const float id2 = 1.0f / (dx * dx + dy * dy + dz * dz);
  const float3 dn = make_float3(dx * id2, dy * id2, dz * id2);  // depth in units of t
  const float m = a.grid_margin;
  float4* box = a.grid_box + size_t(gi) * T;
  float2* dep = a.grid_dep + size_t(gi) * T;
  for (uint32_t c = tid; c < GG; c += kGridThreads) start[c] = 0;
  // pass 1: widened 2D boxes and depth ranges; the extent of the boxes
  float lu = INFINITY, hu = -INFINITY, lv = INFINITY, hv = -INFINITY;
  for (uint32_t t = tid; t < T; t += kGridThreads) {
    const float4 v0 = __ldg(a.tris + 3 * t), e1 = __ldg(a.tris + 3 * t + 1), e2 = __ldg(a.tris + 3 * t + 2);
    const float px[3] = {v0.x, v0.x + e1.x, v0.x + e2.x}, py[3] = {v0.y, v0.y + e1.y, v0.y + e2.y},
                pz[3] = {v0.z, v0.z + e1.z, v0.z + e2.z};
    float pu[3], pv[3], pd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      pu[k] = dot3(px[k], py[k], pz[k], u);
      pv[k] = dot3(px[k], py[k], pz[k], v);
      pd[k] = dot3(px[k], py[k], pz[k], dn);
    }
    const float4 b = make_float4(fmin3(pu[0], pu[1], pu[2]) - m, fmax3(pu[0], pu[1], pu[2]) + m,
                                 fmin3(pv[0], pv[1], pv[2]) - m, fmax3(pv[0], pv[1], pv[2]) + m);
    const float2 dd = make_float2(fmin3(pd[0], pd[1], pd[2]), fmax3(pd[0], pd[1], pd[2]));
    box[t] = b;
    dep[t] = dd;
    tnear[t] = dd.x;
    lu = fminf(lu, b.x); hu = fmaxf(hu, b.y); lv = fminf(lv, b.z); hv = fmaxf(hv, b.w);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lu = fminf(lu, __shfl_xor_sync(kFull, lu, o)); hu = fmaxf(hu, __shfl_xor_sync(kFull, hu, o));
    lv = fminf(lv, __shfl_xor_sync(kFull, lv, o)); hv = fmaxf(hv, __shfl_xor_sync(kFull, hv, o));
  }
  if (lane == 0) { red[0][warp] = lu; red[1][warp] = hu; red[2][warp] = lv; red[3][warp] = hv; }
  __syncthreads();
  lu = red[0][0]; hu = red[1][0]; lv = red[2][0]; hv = red[3][0];
  for (int k = 1; k < kGridThreads / 32; ++k) {
    lu = fminf(lu, red[0][k]); hu = fmaxf(hu, red[1][k]); lv = fminf(lv, red[2][k]); hv = fmaxf(hv, red[3][k]);
  }
  const float iu = float(G) / fmaxf(hu - lu, 1e-30f), iv = float(G) / fmaxf(hv - lv, 1e-30f);
  // pass 2: cell ranges and counts
  for (uint32_t t = tid; t < T; t += kGridThreads) {
    const float4 b = box[t];
    const uint32_t i0 = grid_cell(b.x, lu, iu, G), i1 = grid_cell(b.y, lu, iu, G);
    const uint32_t j0 = grid_cell(b.z, lv, iv, G), j1 = grid_cell(b.w, lv, iv, G);
    tcell[t] = i0 | (i1 << 8) | (j0 << 16) | (j1 << 24);
    for (uint32_t i = i0; i <= i1; ++i)
      for (uint32_t j = j0; j <= j1; ++j) atomicAdd(&start[i * G + j], 1u);
  }
  __syncthreads();
  const uint32_t total = grid_scan(start, GG, wsum);
  for (uint32_t c = tid; c < GG; c += kGridThreads) cur[c] = start[c];
  if (tid == 0) start[GG] = total;
  float4* hdr = a.grid_hdr + 4 * size_t(gi);
  if (total > kGridCap) {  // too many entries: this grid's rays walk the tree
    if (tid == 0) hdr[3] = make_float4(iv, __int_as_float(0), 0.f, 0.f);
    return;
  }
  __syncthreads();
  // pass 3: fill
  for (uint32_t t = tid; t < T; t += kGridThreads) {
    const uint32_t cr = tcell[t];
    const uint32_t i0 = cr & 255, i1 = (cr >> 8) & 255, j0 = (cr >> 16) & 255, j1 = cr >> 24;
    for (uint32_t i = i0; i <= i1; ++i)
      for (uint32_t j = j0; j <= j1; ++j) ent[atomicAdd(&cur[i * G + j], 1u)] = uint16_t(t);
  }
  __syncthreads();
  // pass 4: each cell by (near depth, slot): Shell sort with Ciura's gaps
  for (uint32_t c = tid; c < GG; c += kGridThreads) {
    uint16_t* e = ent + start[c];
    const int n = int(start[c + 1] - start[c]);
    const int gaps[8] = {701, 301, 132, 57, 23, 10, 4, 1};
    for (int gk = 0; gk < 8; ++gk) {
      const int gap = gaps[gk];
      for (int i = gap; i < n; ++i) {
        const uint16_t x = e[i];
        const float kx = tnear[x];
        int j = i;
        while (j >= gap) {
          const uint16_t y = e[j - gap];
          const float ky = tnear[y];
          if (ky < kx || (ky == kx && y < x)) break;
          e[j] = y;
          j -= gap;
        }
        e[j] = x;
      }
    }
  }
  __syncthreads();
  // pass 5: out
  uint32_t* cells = a.grid_cells + size_t(gi) * (GG + 1);
  for (uint32_t c = tid; c <= GG; c += kGridThreads) cells[c] = start[c];
  uint16_t* eo = a.grid_ent + size_t(gi) * kGridCap;
  for (uint32_t k = tid; k < total; k += kGridThreads) eo[k] = ent[k];
  if (tid == 0) {
    hdr[0] = make_float4(u.x, u.y, u.z, lu);
    hdr[1] = make_float4(v.x, v.y, v.z, lv);
    hdr[2] = make_float4(dn.x, dn.y, dn.z, iu);
    hdr[3] = make_float4(iv, __int_as_float(1), 0.f, 0.f);
  }
}

void launch_grid_build(const TraceArgs& a, cudaStream_t s) {
  if (!a.grid_hdr || a.ntris == 0) return;
  static std::atomic<uint64_t> opted{0};
  smem_opt_in(k_grid_build, int(grid_build_smem(32, kGridMaxTris)), opted);  // the largest launch
  const size_t smem = grid_build_smem(a.grid_g, a.ntris);
  k_grid_build<<<a.S + 1, kGridThreads, smem, s>>>(a);
}

// A lane's walk through one grid cell: the cell's entry range [e, e1), the
// ray's 2D point and depth, and the next entry's triangle (loaded a step
// ahead, so a step's depth-range, box and next-entry loads go out together).
struct GridWalk {
  uint32_t e = 0, e1 = 0, gi = 0, nt = 0;
  float pu = 0.f, pv = 0.f, pd = 0.f;
};

// Sets up the walk of L's current ray through grid gi; false when the grid
// overflowed or the origin is beyond grid_far (the caller walks the tree).
__device__ __forceinline__ bool grid_setup(const TraceArgs& a, uint32_t gi, const LaneRay& L, GridWalk& g) {
  const float4 h3 = __ldg(a.grid_hdr + 4 * gi + 3);
  const float ox = L.ray.ox, oy = L.ray.oy, oz = L.ray.oz;
  if (__float_as_int(h3.y) == 0 || fmax3(fabsf(ox), fabsf(oy), fabsf(oz)) > a.grid_far) return false;
  const float4 h0 = __ldg(a.grid_hdr + 4 * gi), h1 = __ldg(a.grid_hdr + 4 * gi + 1),
               h2 = __ldg(a.grid_hdr + 4 * gi + 2);
  const uint32_t G = a.grid_g;
  g.gi = gi;
  g.pu = dot3(ox, oy, oz, make_float3(h0.x, h0.y, h0.z));
  g.pv = dot3(ox, oy, oz, make_float3(h1.x, h1.y, h1.z));
  g.pd = dot3(ox, oy, oz, make_float3(h2.x, h2.y, h2.z));
  const uint32_t c = grid_cell(g.pu, h0.w, h2.w, G) * G + grid_cell(g.pv, h1.w, h3.x, G);
  const uint32_t* cells = a.grid_cells + size_t(gi) * (G * G + 1);
  g.e = __ldg(cells + c);
  g.e1 = __ldg(cells + c + 1);
  if (g.e < g.e1) g.nt = __ldg(a.grid_ent + size_t(gi) * kGridCap + g.e);
  return true;
}

// One entry of the walk (shadow walks: any hit in (0, L.tb); primary walks:
// nearest hit beyond tmin with the tie rule); g.e = g.e1 when the walk is over.
template <bool COUNT>
__device__ __forceinline__ void grid_step(const TraceArgs& a, LaneRay& L, GridWalk& g, Work& w) {
  const uint32_t t = VLB_CLAMP(g.nt, a.ntris, a.err), T = a.ntris;
  const float2 dd = __ldg(a.grid_dep + size_t(g.gi) * T + t);
  const float4 b = __ldg(a.grid_box + size_t(g.gi) * T + t);
  if (g.e + 1 < g.e1) g.nt = __ldg(a.grid_ent + size_t(g.gi) * kGridCap + VLB_CLAMP(g.e + 1, kGridCap, a.err));
  ++g.e;
  if constexpr (COUNT) { ++w.wnodes; ++w.lnodes; }
  const float tlo = L.shadow ? 0.0f : a.tmin, m = a.grid_margin;
  if (dd.y - g.pd + m <= tlo) return;                                   // ends before the interval
  if (dd.x - g.pd - m > prune_limit(L.tb)) { g.e = g.e1; return; }      // this and every later entry too far
  if (g.pu < b.x || g.pu > b.y || g.pv < b.z || g.pv > b.w) return;
  if constexpr (COUNT) ++w.wtris;
  const float4 v0 = __ldg(a.tris + 3 * t), e1 = __ldg(a.tris + 3 * t + 1), e2 = __ldg(a.tris + 3 * t + 2);
  const float th = tri_hit(L.ray, v0, e1, e2);
  if (!(th > tlo)) return;
  if (L.shadow) {
    if (th < L.tb) { L.slot = int(t); g.e = g.e1; }
    return;
  }
  const int tid = __float_as_int(v0.w);
  if (th < L.tb || (th == L.tb && L.slot >= 0 && tid < L.id)) { L.tb = th; L.slot = int(t); L.id = tid; }
}

// Starts the current walk of L (primary: grid L.s; shadow: grid S).  Where
// the grid cannot take the ray, the tree walk runs to its end here and the
// grid walk is left empty.
template <bool COUNT>
__device__ __forceinline__ void grid_begin(const TraceArgs& a, LaneRay& L, GridWalk& g, Work& w) {
  const uint32_t gi = L.shadow ? a.S : L.s;
  if (grid_setup(a, gi, L, g)) return;
  g.e = g.e1 = 0;
  bool active = true;
  const float dx = L.shadow ? a.sun.x : L.d.x, dy = L.shadow ? a.sun.y : L.d.y, dz = L.shadow ? a.sun.z : L.d.z;
  if (L.shadow)
    traverse<true, COUNT, true>(octant_of(dx, dy, dz), L.ray, active, a.nodes, a.tris, a.ntris, 0.0f, L.tb, L.slot,
                                L.id, a.err, w);
  else
    traverse<false, COUNT, true>(octant_of(dx, dy, dz), L.ray, active, a.nodes, a.tris, a.ntris, a.tmin, L.tb,
                                 L.slot, L.id, a.err, w);
}

constexpr int kGridSteps = 8;  // entry steps per turn

// Persistent warps; each lane runs its rays through a small state machine --
// primary cell walk, shading, shadow cell walk, tile entries -- and idle
// lanes refill together from the ray counter (as k_trace_dyn, but numbered
// direction-major: rays fetched together share a direction, hence a grid, and
// are Morton-neighbour probes).
template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads) k_trace_grid(const TraceArgs a) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t P = (a.nprobes + 31) / 32 * 32;
  const uint32_t R = P * a.S;
  Work w;
  LaneRay L;
  GridWalk g;
  make_ray(L.ray, 0.f, 0.f, 0.f, 1.f, 1.f, 1.f);
  bool exhausted = false;
  for (;;) {
    const unsigned idle = __ballot_sync(kFull, !L.has);
    if (!exhausted && (idle == kFull || __popc(idle) >= kRefillIdle)) {
      const int leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (int(lane) == leader) base = atomicAdd(a.work_counter, uint32_t(__popc(idle)));
      base = __shfl_sync(kFull, base, leader);
      if (base >= R) exhausted = true;
      if (!L.has) {
        const uint32_t r = base + __popc(idle & lane_lt_mask());
        if (r < R) {
          const uint32_t t = r / P, sl = r - t * P;
          if (sl < a.nprobes) {
            lr_start(a, L, a.order[sl], __ldg(a.dir_order + t));
            grid_begin<COUNT>(a, L, g, w);
          }
        }
      }
    }
    if (!__any_sync(kFull, L.has)) {
      if (exhausted) break;
      continue;
    }
#pragma unroll 1
    for (int k = 0; k < kGridSteps; ++k) {
      const bool walking = L.has && g.e < g.e1;
      if (!__any_sync(kFull, walking)) break;
      if (walking) grid_step<COUNT>(a, L, g, w);
    }
    if (!L.has || g.e < g.e1) continue;
    Shaded o;
    if (!lr_finish<COUNT>(a, L, o, w)) {  // a lit hit: its shadow walk
      grid_begin<COUNT>(a, L, g, w);
      continue;
    }
    L.has = false;
    emit_tile(a, L, o);
  }
  if constexpr (COUNT) {
    atomicAdd(a.counters + 0, (unsigned long long)w.wnodes);
    atomicAdd(a.counters + 1, (unsigned long long)w.wtris);
    atomicAdd(a.counters + 2, (unsigned long long)w.shadow);
    atomicAdd(a.counters + 3, (unsigned long long)w.lnodes);
  }
}

template <bool COUNT>
static void launch_grid_trace(const TraceArgs& a, int num_sms, cudaStream_t s) {
  static int per_sm = 0;
  if (!per_sm) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_grid<COUNT>, kTraceThreads, 0);
    if (per_sm < 1) per_sm = 1;
  }
  const uint64_t rays = uint64_t((a.nprobes + 31) / 32 * 32) * a.S;
  const uint64_t ctas = std::min<uint64_t>((rays + kTraceThreads - 1) / kTraceThreads, uint64_t(num_sms) * per_sm);
  k_trace_grid<COUNT><<<uint32_t(std::max<uint64_t>(ctas, 1)), kTraceThreads, 0, s>>>(a);
}

bool grid_supported(uint32_t ntris, uint32_t nprobes, uint32_t S) {
  return ntris > 0 && ntris <= kGridMaxTris && uint64_t((nprobes + 31) / 32 * 32) * S < (1ull << 31);
}

void launch_trace_tile(const TraceArgs& a, int num_sms, cudaStream_t s) {
  if (a.grid_hdr) {
    if (a.counters) launch_grid_trace<true>(a, num_sms, s);
    else launch_grid_trace<false>(a, num_sms, s);
    return;
  }
  if (trace_dyn_supported(a)) {
    if (a.shading == VLB_SHADE_REF_PHONG) {  // the wide tree is not built into these: the binary walk
      if (a.counters) launch_dyn<true, false, true>(a, num_sms, s);
      else launch_dyn<false, false, true>(a, num_sms, s);
    } else if (a.wnodes) {
      if (a.counters) launch_dyn<true, true, false>(a, num_sms, s);
      else launch_dyn<false, true, false>(a, num_sms, s);
    } else {
      if (a.counters) launch_dyn<true, false, false>(a, num_sms, s);
      else launch_dyn<false, false, false>(a, num_sms, s);
    }
    return;
  }
  if (a.counters) launch<0, 1, true>(a, num_sms, s);
  else launch<0, 1, false>(a, num_sms, s);
}

// Batched bake: the same packet tracing, with work items numbered across all
// jobs (job j owns items [item_begin, item_begin + packets * chunks)); a warp
// finds its job by binary search over the item ranges and traces that job's
// scene.  Radiance goes to the job's rows of its direction set's tile.
__device__ __forceinline__ void batch_emit(const BakeJobDev& j, uint32_t p, uint32_t s, const Shaded& o) {
  if (!VLB_INB(p, j.nprobes, j.err) || !VLB_INB(s, j.S, j.err)) return;
  const size_t row = size_t(p) * 3;
  if (j.radiance) {
    j.radiance[row * j.S + s] = o.r;
    j.radiance[(row + 1) * j.S + s] = o.g;
    j.radiance[(row + 2) * j.S + s] = o.b;
  } else {
    store_bf16(j.radiance_bf16, row, j.S, s, o.r, j.bf16_split);
    store_bf16(j.radiance_bf16, row + 1, j.S, s, o.g, j.bf16_split);
    store_bf16(j.radiance_bf16, row + 2, j.S, s, o.b, j.bf16_split);
  }
}

// Batched bake.  Job j owns the rays [ray_begin, ray_begin + P*S) of one
// numbering over all jobs (P: its probe count rounded up to 32; ray r of a job
// is probe slot r / S, direction position r % S), each job's range rounded up
// to whole chunks of 32 * chunk_lanes rays.  A warp takes a chunk from the
// counter (one atomic), finds its job by binary search over the ranges, and
// hands the chunk's next 32 rays to its lanes whenever all of them are idle;
// every lane runs its ray through its own state machine (lr_*), and the job's
// fields stay warp-uniform.  Kept hits are
// written after the primary walk; a relight starts from the kept hit with only
// its shadow walk.  Every job walks per lane: results do not depend on the
// traversal mode.
template <bool REF>
__global__ void __launch_bounds__(kTraceThreads, 8) k_trace_batch(const BakeJobDev* __restrict__ jobs, uint32_t njobs,
                                                               uint32_t total, uint32_t chunk, uint32_t* counter) {
  const uint32_t lane = threadIdx.x & 31;
  Work w;
  int stack[kLaneStack];
  LaneRay L;
  make_ray(L.ray, 0.f, 0.f, 0.f, 1.f, 1.f, 1.f);
  for (;;) {
    uint32_t c = 0;
    if (lane == 0) c = atomicAdd(counter, chunk);
    c = __shfl_sync(kFull, c, 0);
    if (c >= total) break;
    uint32_t lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (__ldg(&jobs[mid].ray_begin) <= c) lo = mid; else hi = mid - 1;
    }
    const BakeJobDev& j = jobs[lo];
    const uint32_t P = (j.nprobes + 31) / 32 * 32;
    const uint32_t R = P * j.S;
    uint32_t r0 = c - j.ray_begin;                // the chunk's first ray in the job
    const uint32_t r1 = min(R, r0 + chunk);       // end of its real rays (the rest is padding)
    for (;;) {
      const unsigned idle = __ballot_sync(kFull, !L.has);
      // a whole idle warp takes the chunk's next rays, in lane order: its rays
      // start together and share their nodes (as in k_trace_dyn; measured 11 %
      // faster on the 256-job batch than refilling any idle lane)
      if (idle == kFull && r0 < r1) {
        const uint32_t r = r0 + __popc(idle & lane_lt_mask());
        r0 = min(r1, r0 + uint32_t(__popc(idle)));
        if (!L.has && r < r1) {
          const uint32_t sl = r / j.S, t = r - sl * j.S;
          if (sl < j.nprobes) {
            const uint32_t p = j.order[sl];
            lr_start(j, L, p, __ldg(j.dir_order + t));
            if (j.hits_in) {  // relight: the kept primary hit, only the shadow walk remains
              const int2 h = __ldg(j.hits_in + size_t(p) * j.S + L.s);
              L.slot = h.x;
              L.tb = __int_as_float(h.y);
              L.id = h.x >= 0 ? __float_as_int(__ldg(j.tris + 3 * VLB_CLAMP(h.x, j.ntris, j.err)).w) : -1;
              Shaded o;
              if (lr_finish<false, BakeJobDev, REF>(j, L, o, w)) {
                L.has = false;
                batch_emit(j, L.p, L.s, o);
              }
            }
          }
        }
      }
      if (!__any_sync(kFull, L.has)) {
        if (r0 >= r1) break;
        continue;
      }
      // one while-while turn, as in k_trace_dyn (the octant-specialised node
      // phase measured 4 % slower here, also when only jobs of 1024
      // directions take it: its eight copies cost this kernel more than they
      // save)
      lr_node_steps<false, BakeJobDev, false, true, -1>(j, L, stack, w, kNodeSteps);
      lr_park(L, stack);
      if (!L.has) continue;
      if (L.leaf >= 0) lr_leaf<false>(j, L, w);
      if (L.cur != kWalkEnd) continue;
      if (!L.shadow && j.hits_out) j.hits_out[size_t(L.p) * j.S + L.s] = make_int2(L.slot, __float_as_int(L.tb));
      Shaded o;
      if (!lr_finish<false, BakeJobDev, REF>(j, L, o, w)) continue;
      L.has = false;
      batch_emit(j, L.p, L.s, o);
    }
  }
}

template <bool REF>
static void launch_batch(const BakeJobDev* jobs, uint32_t njobs, uint32_t total_rays, uint32_t chunk,
                         uint32_t* counter, int num_sms, cudaStream_t s) {
  static int per_sm = 0;
  if (!per_sm) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_batch<REF>, kTraceThreads, 0);
    if (per_sm < 1) per_sm = 1;
  }
  const uint64_t ctas = std::min<uint64_t>((uint64_t(total_rays) / chunk + kTraceWarps - 1) / kTraceWarps + 1,
                                           uint64_t(num_sms) * per_sm);
  k_trace_batch<REF><<<uint32_t(ctas), kTraceThreads, 0, s>>>(jobs, njobs, total_rays, chunk, counter);
}

void launch_trace_batch(const BakeJobDev* jobs, uint32_t njobs, uint32_t total_rays, uint32_t chunk,
                        uint32_t* counter, bool ref_shading, int num_sms, cudaStream_t s) {
  if (!total_rays || !njobs) return;
  if (ref_shading) launch_batch<true>(jobs, njobs, total_rays, chunk, counter, num_sms, s);
  else launch_batch<false>(jobs, njobs, total_rays, chunk, counter, num_sms, s);
}

__global__ void k_scatter_rows(const float* __restrict__ src, float* const* __restrict__ dst,
                               const uint32_t* __restrict__ src_probe0, const uint32_t* __restrict__ nprobes,
                               uint32_t K) {
  const uint32_t jb = blockIdx.y;
  const size_t n = size_t(nprobes[jb]) * K * 3;
  const float* sp = src + size_t(src_probe0[jb]) * K * 3;
  float* dp = dst[jb];
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    dp[i] = sp[i];
}

void launch_scatter_rows(const float* src, float* const* dst, const uint32_t* src_probe0, const uint32_t* nprobes,
                         uint32_t njobs, uint32_t K, cudaStream_t s) {
  if (njobs) k_scatter_rows<<<dim3(64, njobs), 256, 0, s>>>(src, dst, src_probe0, nprobes, K);
}

// ---- probe evaluation: the consumer side of a baked grid -------------------------
// Restates shaders/main.rchit:124-168 with shaders/sh.rmiss:23-39 (intended
// math; the reference's grid-origin, probe-index, coefficient-stride and 0/0
// faults are not reproduced).  One thread per shading point: the cell of
// the grid holding the point, its 8 corner probes (gridVertices order: bit 2
// x, bit 1 y, bit 0 z), a visibility ray from point + bias * n toward each
// probe (any hit in (0, |d|), per-lane walk: the rays of a warp share
// nothing), and the distance-weighted mean of the visible probes' SH
// evaluated at the normal.
__device__ __forceinline__ uint32_t ref_grid_index(const uint32_t* cnt, uint32_t i, uint32_t j, uint32_t k) {
  // breadth-first grid order of LightBaker::probePositionsFromBoudingBox
  const uint32_t q = j == 0 ? i : cnt[0] + i * (cnt[1] - 1) + (j - 1);
  return k == 0 ? q : cnt[0] * cnt[1] + q * (cnt[2] - 1) + (k - 1);
}

template <int LMAX>
__global__ void __launch_bounds__(128) k_probe_eval(const ProbeEvalArgs a) {
  constexpr int K = sh_k<LMAX>();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  float x[3], nv[3];
  for (int c = 0; c < 3; ++c) {
    x[c] = a.points[3 * size_t(i) + c];
    nv[c] = a.normals[3 * size_t(i) + c];
  }
  const float rn = rsqrtf(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
  for (float& c : nv) c *= rn;
  float Y[16];
  sh_basis<LMAX>(nv[0], nv[1], nv[2], Y);
  const float o[3] = {fmaf(a.bias, nv[0], x[0]), fmaf(a.bias, nv[1], x[1]), fmaf(a.bias, nv[2], x[2])};
  int cell[3];
  for (int c = 0; c < 3; ++c) {
    const int hi = max(int(a.counts[c]) - 2, 0);
    cell[c] = hi == 0 ? 0 : min(max(int(floorf(__fdiv_rn(__fsub_rn(x[c], a.org[c]), a.step[c]))), 0), hi);
  }
  const float wmax = sqrtf(a.step[0] * a.step[0] + a.step[1] * a.step[1] + a.step[2] * a.step[2]);
  float sum[3] = {0.f, 0.f, 0.f}, ws = 0.f;
  uint32_t mask = 0;
  Work w;
  for (int c = 0; c < 8; ++c) {
    uint32_t ijk[3];
    float d[3];
    for (int e = 0; e < 3; ++e) {
      ijk[e] = min(uint32_t(cell[e]) + ((uint32_t(c) >> (2 - e)) & 1u), a.counts[e] - 1);
      const float p = __fadd_rn(a.org[e], __fmul_rn(a.step[e], float(ijk[e])));
      d[e] = p - x[e];
    }
    const float t = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    bool visible = true;
    if (t > 0.f && a.ntris) {
      const float it = 1.0f / t;
      const float dx = d[0] * it, dy = d[1] * it, dz = d[2] * it;
      RayCtx ray;
      make_ray(ray, o[0], o[1], o[2], dx, dy, dz);
      bool act = true;
      float tb = t;
      int slot = -1, id = -1;
      traverse<true, false, true>(octant_of(dx, dy, dz), ray, act, a.nodes, a.tris, a.ntris, 0.0f, tb, slot, id,
                                  a.err, w);
      visible = slot < 0;
    }
    if (!visible) continue;
    mask |= 1u << c;
    const float wc = wmax - t;
    const float* cp = a.coeffs + size_t(ref_grid_index(a.counts, ijk[0], ijk[1], ijk[2])) * K * 3;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      float e = 0.f;
#pragma unroll
      for (int k = 0; k < K; ++k) e = fmaf(__ldg(cp + 3 * k + ch), Y[k], e);
      sum[ch] = fmaf(wc, e, sum[ch]);
    }
    ws += wc;
  }
  for (int ch = 0; ch < 3; ++ch) a.out[3 * size_t(i) + ch] = ws > 0.f ? sum[ch] / ws : 0.f;
  if (a.vis) a.vis[i] = uint8_t(mask);
}

void launch_probe_eval(const ProbeEvalArgs& a, uint32_t lmax, cudaStream_t s) {
  if (!a.n) return;
  const uint32_t g = (a.n + 127) / 128;
  if (lmax == 3) k_probe_eval<3><<<g, 128, 0, s>>>(a);
  else k_probe_eval<2><<<g, 128, 0, s>>>(a);
}

void launch_trace_fused(const TraceArgs& a, int num_sms, cudaStream_t s) {
  if (a.K == 9) launch<1, 9, false>(a, num_sms, s);
  else launch<1, 16, false>(a, num_sms, s);
}

}  // namespace vlbk
