// k_trace_fused.cu -- the bake in one kernel: per-lane traversal, shading and
// the SH projection of shaders/sh.comp:23-42, with no radiance tile.
//
// Work items.  Item (job, probe, chunk c) is the probe's rays at positions
// [c*D, min(S, (c+1)*D)) of the direction set's trace order (grouped by
// octant, then by position on the octant's face); D = fused_chunk_rays(S),
// a function of S alone.  Items are numbered probe-major over the job's
// Morton-sorted probes, so neighbouring items share a probe or a Morton
// neighbour.  Persistent warps take items from one counter.
//
// Sub-batches.  A warp cuts its items into sub-batches of up to kSubRays rays
// and keeps up to kSubBufs in flight in a shared-memory ring (the RGB of each
// ray).  Idle lanes take the oldest sub-batch's unissued rays first, then the
// next one's, so lanes that finish early run ahead into the
// next sub-batch (or the next item) while others finish their walks: a warp
// waits for a slow ray only when kSubBufs sub-batches are behind it.  Each lane
// runs the per-lane state machine of the lane walk (primary walk, shading,
// shadow walk) and writes its ray's RGB into the ring when done.  As in the
// tile lane walk, a warp does this bookkeeping only when enough of its lanes
// are idle; the turns in between are pure traversal.
//
// Projection.  When the oldest sub-batch is complete the warp projects it:
// output v = 3k + ch (lane v, and lane v - 32 for v >= 32) sums
// basis16[s_i][k] * L_i[ch] over the sub-batch's rays i in ray order in FP32
// and adds that sum to the item's FP64 running sum.  After the item's last
// sub-batch the item sum goes to the output (one chunk per probe) or to an
// FP32 partial; the chunk that finishes a probe last (atomic ticket) adds the
// probe's partials in FP64 in chunk order.  Every sum has a fixed order, so a
// probe's coefficients do not depend on the warp, the lane, the timing or the
// other jobs of a batch.
#include "trace_common.cuh"

#include <algorithm>
#include <atomic>

namespace vlbk {

constexpr int kSubRays = 32;
constexpr int kSubBufs = 2;
constexpr uint32_t kSubFirst = 1, kSubLast = 2;

// One sub-batch in flight.
struct SubBatch {
  uint32_t job, p, c, t0;
  uint32_t cnt, issued, fin, flags;
};

// Per-warp shared state.  Everything but the lanes' own rays is warp-uniform
// and lives here, not in registers (the trace walk needs them): written by
// lane 0 only, read by every lane after a __syncwarp.
template <int V>
struct FusedWarp {
  float rad[kSubBufs][3][kSubRays];    // RGB of each ray, channel-major
  SubBatch q[kSubBufs];
  double acc[V];                       // the current item's running FP64 sums, output v at acc[v]
  uint32_t head, n;                    // ring: oldest slot, sub-batches in flight
  uint32_t ij, ip, ic, itn, ite, it0;  // the item being cut: job, probe, chunk, next/end/first ray
  uint32_t have_item, exhausted;
};

template <bool MULTI>
__device__ __forceinline__ const BakeJobDev& job_of(const BakeJobDev* jobs, const BakeJobDev& one, uint32_t j) {
  if constexpr (MULTI) return jobs[j];
  else return one;
}

// The job owning work item `it` (binary search over item_begin).
__device__ __forceinline__ uint32_t find_job(const BakeJobDev* __restrict__ jobs, uint32_t njobs, uint32_t it) {
  uint32_t lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (__ldg(&jobs[mid].item_begin) <= it) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Projects the complete sub-batch at the ring's head into the item's running
// sums and, after the item's last sub-batch, writes the item (output or
// partial, and the probe's FP64 chunk sum when its last chunk is done).
template <int K, bool MULTI>
__device__ __forceinline__ void retire_head(FusedWarp<3 * K>& fw, const BakeJobDev* __restrict__ jobs,
                                            const BakeJobDev& one, uint32_t lane) {
  constexpr int V = 3 * K;
  const uint32_t e = fw.head;
  const SubBatch q = fw.q[e];
  const BakeJobDev& J = job_of<MULTI>(jobs, one, q.job);
  const uint32_t* dord = J.dir_order + q.t0;
  for (int v = int(lane); v < V; v += 32) {
    const int k = v / 3, ch = v - 3 * k;
    float s = 0.f;
#pragma unroll 4
    for (uint32_t i = 0; i < q.cnt; ++i)
      s = fmaf(__ldg(J.basis16 + size_t(VLB_CLAMP(__ldg(dord + i), J.S, J.err)) * 16 + k), fw.rad[e][ch][i], s);
    fw.acc[v] = ((q.flags & kSubFirst) ? 0.0 : fw.acc[v]) + double(s);
  }
  if ((q.flags & kSubLast) && VLB_INB(q.p, J.nprobes, J.err) && VLB_INB(q.c, J.chunks, J.err)) {
    float* dst = J.chunks == 1 ? J.out + size_t(q.p) * V : J.partial + (size_t(q.p) * J.chunks + q.c) * V;
    for (int v = int(lane); v < V; v += 32) dst[v] = float(fw.acc[v]);
    if (J.chunks > 1) {
      __threadfence();
      __syncwarp();
      uint32_t ticket = 0;
      if (lane == 0) ticket = atomicAdd(J.done + q.p, 1u);
      ticket = __shfl_sync(kFull, ticket, 0);
      if (ticket == J.chunks - 1) {  // the probe's last chunk: FP64 sum in chunk order
        __threadfence();
        const float* src = J.partial + size_t(q.p) * J.chunks * V;
        for (int v = int(lane); v < V; v += 32) {
          double t = 0.0;
          for (uint32_t c = 0; c < J.chunks; ++c) t += double(__ldcg(src + size_t(c) * V + v));
          J.out[size_t(q.p) * V + v] = float(t);
        }
      }
    }
  }
  __syncwarp();
  if (lane == 0) {
    fw.head = (e + 1) % kSubBufs;
    fw.n -= 1;
  }
  __syncwarp();
}

// Appends the next sub-batch (of the current item, or of a new item from the
// counter) to the ring while there is room and the newest one has handed out
// all its rays.
template <bool MULTI, class FW>
__device__ __forceinline__ void fill_ring(FW& fw, const BakeJobDev* __restrict__ jobs, const BakeJobDev& one,
                                          uint32_t njobs, uint32_t total, uint32_t* counter, uint32_t lane) {
  while (fw.n < kSubBufs) {
    const uint32_t n = fw.n;
    if (n > 0) {
      const SubBatch& t = fw.q[(fw.head + n - 1) % kSubBufs];
      if (t.issued < t.cnt) break;  // the newest still has rays to hand out
    }
    if (!fw.have_item) {
      if (fw.exhausted) break;
      uint32_t it = 0;
      if (lane == 0) it = atomicAdd(counter, 1u);
      it = __shfl_sync(kFull, it, 0);
      if (it >= total) {
        if (lane == 0) fw.exhausted = 1;
        __syncwarp();
        break;
      }
      const uint32_t j = MULTI ? find_job(jobs, njobs, it) : 0;
      const BakeJobDev& J = job_of<MULTI>(jobs, one, j);
      const uint32_t loc = it - J.item_begin;
      uint32_t slot, c;
      if (J.chunk_major) {
        c = loc / J.nprobes;
        slot = loc - c * J.nprobes;
      } else {
        slot = loc / J.chunks;
        c = loc - slot * J.chunks;
      }
      const uint32_t p = VLB_CLAMP(J.order[VLB_CLAMP(slot, J.nprobes, J.err)], J.nprobes, J.err);
      __syncwarp();
      if (lane == 0) {
        fw.ij = j; fw.ip = p; fw.ic = c;
        fw.it0 = fw.itn = c * J.chunk_rays;
        fw.ite = min(J.S, c * J.chunk_rays + J.chunk_rays);
        fw.have_item = 1;
      }
      __syncwarp();
    }
    const uint32_t itn = fw.itn, ite = fw.ite;
    const uint32_t cnt = min(ite - itn, uint32_t(kSubRays));
    __syncwarp();
    if (lane == 0) {
      SubBatch& q = fw.q[(fw.head + n) % kSubBufs];
      q.job = fw.ij; q.p = fw.ip; q.c = fw.ic; q.t0 = itn; q.cnt = cnt; q.issued = 0; q.fin = 0;
      q.flags = (itn == fw.it0 ? kSubFirst : 0u) | (itn + cnt == ite ? kSubLast : 0u);
      fw.itn = itn + cnt;
      if (itn + cnt >= ite) fw.have_item = 0;
      fw.n = n + 1;
    }
    __syncwarp();
  }
}

// A finished ray: its RGB into the ring, and the per-ray debug arrays.
template <class FW>
__device__ __forceinline__ void store_ray(FW& fw, const BakeJobDev& J, const LaneRay& L, const Shaded& o,
                                          uint32_t lslot) {
  const uint32_t le = lslot >> 8, lpos = lslot & 255;
  if (!VLB_INB(le, kSubBufs, J.err) || !VLB_INB(lpos, kSubRays, J.err)) return;
  fw.rad[le][0][lpos] = o.r;
  fw.rad[le][1][lpos] = o.g;
  fw.rad[le][2][lpos] = o.b;
  if (J.hit_tri || J.shadow || J.dbg_radiance) {
    const size_t ri = size_t(L.p) * J.S + L.s;
    if (J.hit_tri) J.hit_tri[ri] = o.tri;
    if (J.shadow) J.shadow[ri] = o.vis;
    if (J.dbg_radiance) {
      J.dbg_radiance[3 * ri] = o.r; J.dbg_radiance[3 * ri + 1] = o.g; J.dbg_radiance[3 * ri + 2] = o.b;
    }
  }
}

// MINB: resident CTAs per SM the register allocation is sized for (7, 8 or 9);
// REF: the reference's shading (vlb_shading VLB_SHADE_REF_PHONG).
template <int K, bool MULTI, int MINB, bool REF>
__global__ void __launch_bounds__(kTraceThreads, MINB) k_trace_fused(const BakeJobDev* __restrict__ jobs,
                                                                     const BakeJobDev one, uint32_t njobs,
                                                                     uint32_t total, uint32_t* counter,
                                                                     uint32_t node_steps, uint32_t refill_idle) {
  __shared__ FusedWarp<3 * K> fw_all[kTraceWarps];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  FusedWarp<3 * K>& fw = fw_all[warp];
  if (lane == 0) {
    fw.head = fw.n = 0;
    fw.have_item = fw.exhausted = 0;
  }
  __syncwarp();
  Work w;
  int stack[kLaneStack];
  LaneRay L;
  make_ray(L.ray, 0.f, 0.f, 0.f, 1.f, 1.f, 1.f);
  uint32_t lslot = 0;  // the lane's ray: ring slot << 8 | position
  for (;;) {
    // Bookkeeping only when enough of the warp is idle, as in the tile lane
    // walk: retire complete sub-batches, refill the ring, hand out rays.
    bool done_now = false;
    unsigned idle = __ballot_sync(kFull, !L.has);
    if (idle == kFull || uint32_t(__popc(idle)) >= refill_idle) {
      while (fw.n > 0 && fw.q[fw.head].fin == fw.q[fw.head].cnt) retire_head<K, MULTI>(fw, jobs, one, lane);
      fill_ring<MULTI>(fw, jobs, one, njobs, total, counter, lane);
      const uint32_t n = fw.n, head = fw.head;
      for (uint32_t k = 0; k < n && idle; ++k) {
        const uint32_t e = (head + k) % kSubBufs;
        const uint32_t issued = fw.q[e].issued, avail = fw.q[e].cnt - issued;
        if (!avail) continue;
        const uint32_t take = min(avail, uint32_t(__popc(idle)));
        const uint32_t rank = __popc(idle & lane_lt_mask());
        if (((idle >> lane) & 1u) && rank < take) {
          const uint32_t pos = issued + rank;
          const BakeJobDev& J = job_of<MULTI>(jobs, one, fw.q[e].job);
          const uint32_t s = __ldg(J.dir_order + fw.q[e].t0 + pos);
          lslot = (e << 8) | pos;
          lr_start(J, L, fw.q[e].p, s);
          if (J.hits_in) {  // relight: the kept primary hit, only the shadow walk remains
            const int2 hk = __ldg(J.hits_in + size_t(L.p) * J.S + s);
            L.slot = hk.x;
            L.tb = __int_as_float(hk.y);
            L.id = hk.x >= 0 ? __float_as_int(__ldg(J.tris + 3 * VLB_CLAMP(hk.x, J.ntris, J.err)).w) : -1;
            Shaded o;
            if (lr_finish<false, BakeJobDev, REF>(J, L, o, w)) {
              L.has = false;
              done_now = true;
              store_ray(fw, J, L, o, lslot);
            }
          }
        }
        __syncwarp();
        if (lane == 0) fw.q[e].issued = issued + take;
        idle = __ballot_sync(kFull, !L.has && !done_now);
        __syncwarp();
      }
      if (fw.n == 0 && fw.exhausted) break;  // nothing in flight, nothing left
    }
    if (__any_sync(kFull, L.has)) {
      const BakeJobDev& J = job_of<MULTI>(jobs, one, fw.q[lslot >> 8].job);
      // one while-while turn (as k_trace_dyn): node phase, then leaf phase
      // (the octant-specialised node phase gained nothing here)
      lr_node_steps<false, BakeJobDev, false, !MULTI, -1>(J, L, stack, w, node_steps);
      lr_park(L, stack);
      if (L.has) {
        if (L.leaf >= 0) lr_leaf<false>(J, L, w);
        if (L.cur == kWalkEnd) {
          if (!L.shadow && J.hits_out)
            J.hits_out[size_t(L.p) * J.S + L.s] = make_int2(L.slot, __float_as_int(L.tb));
          Shaded o;
          if (lr_finish<false, BakeJobDev, REF>(J, L, o, w)) {
            L.has = false;
            done_now = true;
            store_ray(fw, J, L, o, lslot);
          }
        }
      }
    }
    // count the finished rays per sub-batch (their RGB is in the ring already)
    unsigned fm = __ballot_sync(kFull, done_now);
    if (!fm) continue;
    const uint32_t le = lslot >> 8;
    while (fm) {
      const int leader = __ffs(fm) - 1;
      const uint32_t e = __shfl_sync(kFull, le, leader);
      const unsigned same = __ballot_sync(kFull, done_now && le == e);
      if (lane == 0) fw.q[e].fin += __popc(same);
      fm &= ~same;
    }
    __syncwarp();
  }
}

template <int K, bool MULTI, int MINB, bool REF>
static void launch_k(const BakeJobDev* jobs, const BakeJobDev& one, uint32_t njobs, uint32_t total,
                     uint32_t* counter, const FusedSched& sc, int num_sms, cudaStream_t s) {
  auto kern = k_trace_fused<K, MULTI, MINB, REF>;
  static int per_sm = 0;
  if (!per_sm) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTraceThreads, 0);
    if (per_sm < 1) per_sm = 1;
  }
  // Shared memory and the L1 cache share one array per SM: ask for no more
  // shared memory than the resident CTAs' rings need, so the walk's node and
  // triangle fetches keep the largest L1 (the carveout is a percentage of the
  // 228 KiB maximum; the hardware rounds it up to a supported size).
  static std::atomic<uint64_t> carved{0};
  {
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0;
    if (bit && !(carved.load(std::memory_order_relaxed) & bit)) {
      const size_t need = sizeof(FusedWarp<3 * K>) * kTraceWarps * size_t(per_sm);
      const int pct = int(std::min<size_t>(100, (need * 100 + 228 * 1024 - 1) / (228 * 1024)));
      cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
      carved.fetch_or(bit, std::memory_order_relaxed);
    }
  }
  const uint64_t ctas = std::min<uint64_t>((uint64_t(total) + kTraceWarps - 1) / kTraceWarps,
                                           uint64_t(num_sms) * per_sm);
  const uint32_t steps = sc.node_steps ? std::min(sc.node_steps, 16u) : 6u;
  const uint32_t refill = sc.refill_idle ? std::min(sc.refill_idle, 32u) : uint32_t(kRefillIdle);
  kern<<<uint32_t(std::max<uint64_t>(ctas, 1)), kTraceThreads, 0, s>>>(jobs, one, njobs, total, counter, steps,
                                                                      refill);
}

template <int K, bool MULTI>
static void launch_occ(const BakeJobDev* jobs, const BakeJobDev& one, uint32_t njobs, uint32_t total,
                       uint32_t* counter, const FusedSched& sc, int num_sms, cudaStream_t s) {
  if (one.shading == VLB_SHADE_REF_PHONG)  // one register budget for the reference shading
    launch_k<K, MULTI, 8, true>(jobs, one, njobs, total, counter, sc, num_sms, s);
  else if (sc.ctas_per_sm == 7) launch_k<K, MULTI, 7, false>(jobs, one, njobs, total, counter, sc, num_sms, s);
  else if (sc.ctas_per_sm == 9) launch_k<K, MULTI, 9, false>(jobs, one, njobs, total, counter, sc, num_sms, s);
  else launch_k<K, MULTI, 8, false>(jobs, one, njobs, total, counter, sc, num_sms, s);
}

void launch_trace_fused_lane(const BakeJobDev* jobs, const BakeJobDev& one, uint32_t njobs, uint32_t total_items,
                             uint32_t K, uint32_t* counter, const FusedSched& sc, int num_sms, cudaStream_t s) {
  if (!total_items || !njobs) return;
  const bool multi = njobs > 1;
  if (K == 16) {
    if (multi) launch_occ<16, true>(jobs, one, njobs, total_items, counter, sc, num_sms, s);
    else launch_occ<16, false>(jobs, one, njobs, total_items, counter, sc, num_sms, s);
  } else {
    if (multi) launch_occ<9, true>(jobs, one, njobs, total_items, counter, sc, num_sms, s);
    else launch_occ<9, false>(jobs, one, njobs, total_items, counter, sc, num_sms, s);
  }
}

}  // namespace vlbk
