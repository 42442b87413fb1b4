// k_ploc.cu -- the traversal BVH: parallel locally-ordered clustering (PLOC,
// Meister and Bittner 2018, "Parallel Locally-Ordered Clustering for Bounding
// Volume Hierarchy Construction") over the Morton-sorted triangles of the LBVH
// build.  Replaces, like the LBVH, the driver's BLAS/TLAS build
// (src/scene_manager.cpp:339-442); the Karras LBVH stays as the exported,
// bit-exact build, this tree is what the trace kernels walk.
//
// Clusters start as the leaves in Morton order.  Each round:
//   1. every cluster finds its nearest neighbour among the R = 16 clusters on
//      either side, distance = surface area of the union box; ties go to the
//      pair with the smaller (|i - j|, parity of the lower index, lower
//      index) -- a symmetric total order on pairs, so the globally closest
//      pair is always mutual and every round merges at least once, and equal
//      neighbours pair up as (2k, 2k+1) instead of one pair per round;
//   2. mutual nearest neighbours merge into a new internal node (the lower
//      index creates it);
//   3. the surviving clusters are compacted in order (an exclusive scan).
// Internal node ids are handed out from n-2 downwards in creation order, so
// the last merge -- the root -- is node 0.  Every step is deterministic: the
// same triangles give the same tree.
#include <algorithm>
#include <vector>

#include "vlb_internal.h"

namespace vlbk {

constexpr int kPlocR = 16;
constexpr int kPlocT = 256;
constexpr int kScanT = 256, kScanPer = 4, kScanTile = kScanT * kScanPer;

__device__ __forceinline__ float union_half_area(const float* a, const float* b) {
  const float dx = fmaxf(a[3], b[3]) - fminf(a[0], b[0]);
  const float dy = fmaxf(a[4], b[4]) - fminf(a[1], b[1]);
  const float dz = fmaxf(a[5], b[5]) - fminf(a[2], b[2]);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx));
}

__global__ void __launch_bounds__(kPlocT) k_ploc_nn(const float* __restrict__ cbox, uint32_t m,
                                                    int32_t* __restrict__ nn) {
  __shared__ float sb[(kPlocT + 2 * kPlocR) * 6];
  const int base = int(blockIdx.x) * kPlocT - kPlocR;
  for (int t = threadIdx.x; t < (kPlocT + 2 * kPlocR) * 6; t += kPlocT) {
    const int g = base + t / 6;
    sb[t] = (g >= 0 && g < int(m)) ? cbox[size_t(g) * 6 + t % 6] : 0.f;
  }
  __syncthreads();
  const int i = int(blockIdx.x) * kPlocT + threadIdx.x;
  if (i >= int(m)) return;
  const float* bi = sb + (threadIdx.x + kPlocR) * 6;
  float best = INFINITY;
  int bj = -1;
  for (int o = -kPlocR; o <= kPlocR; ++o) {
    const int j = i + o;
    if (o == 0 || j < 0 || j >= int(m)) continue;
    const float d = union_half_area(bi, sb + (threadIdx.x + kPlocR + o) * 6);
    bool take = d < best;
    if (!take && d == best) {  // tie: the pair with the smaller (|i-j|, parity of min, min)
      const int g1 = abs(i - j), g2 = abs(i - bj), lo1 = min(i, j), lo2 = min(i, bj);
      take = g1 < g2 || (g1 == g2 && ((lo1 & 1) < (lo2 & 1) || ((lo1 & 1) == (lo2 & 1) && lo1 < lo2)));
    }
    if (take) { best = d; bj = j; }
  }
  nn[i] = bj;
}

// flags[i] = keep << 32 | make: keep unless the lower partner of a mutual
// pair absorbs it; make when i creates the merged node.
__global__ void k_ploc_flags(const int32_t* __restrict__ nn, uint32_t m, uint64_t* __restrict__ flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int j = nn[i];
  const bool mutual = j >= 0 && nn[j] == int(i);
  const uint64_t make = mutual && int(i) < j ? 1 : 0;
  const uint64_t keep = mutual && int(i) > j ? 0 : 1;
  flags[i] = (keep << 32) | make;
}

// Exclusive scan of u64 values in tiles of kScanTile; tile totals to sums.
__global__ void __launch_bounds__(kScanT) k_scan_tiles(const uint64_t* __restrict__ in, uint32_t m,
                                                        uint64_t* __restrict__ out, uint64_t* __restrict__ sums) {
  __shared__ uint64_t s[kScanT];
  const uint32_t t0 = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  uint64_t v[kScanPer], run = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    v[k] = t0 + k < m ? in[t0 + k] : 0;
    run += v[k];
  }
  s[threadIdx.x] = run;
  __syncthreads();
  for (int off = 1; off < kScanT; off <<= 1) {  // Hillis-Steele inclusive scan of the thread totals
    const uint64_t x = threadIdx.x >= unsigned(off) ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += x;
    __syncthreads();
  }
  uint64_t acc = s[threadIdx.x] - run;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    if (t0 + k < m) out[t0 + k] = acc;
    acc += v[k];
  }
  if (threadIdx.x == kScanT - 1) sums[blockIdx.x] = s[threadIdx.x];
}

// One CTA: exclusive scan of the tile totals in place; the grand total to *total.
__global__ void __launch_bounds__(1024) k_scan_sums(uint64_t* __restrict__ sums, uint32_t nb,
                                                     uint64_t* __restrict__ total) {
  __shared__ uint64_t s[1024];
  const uint32_t per = (nb + 1023) / 1024, b0 = threadIdx.x * per;
  uint64_t run = 0;
  for (uint32_t k = 0; k < per && b0 + k < nb; ++k) run += sums[b0 + k];
  s[threadIdx.x] = run;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const uint64_t x = threadIdx.x >= unsigned(off) ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += x;
    __syncthreads();
  }
  uint64_t acc = s[threadIdx.x] - run;
  for (uint32_t k = 0; k < per && b0 + k < nb; ++k) {
    const uint64_t x = sums[b0 + k];
    sums[b0 + k] = acc;
    acc += x;
  }
  if (threadIdx.x == 1023) *total = s[1023];
}

// Merge the mutual pairs and compact, using the scanned flags.
__global__ void k_ploc_merge(const int32_t* __restrict__ cref, const float* __restrict__ cbox,
                             const int32_t* __restrict__ nn, const uint64_t* __restrict__ flags,
                             const uint64_t* __restrict__ scanned, const uint64_t* __restrict__ sums, uint32_t m,
                             int32_t next_id, int32_t* __restrict__ cref_out, float* __restrict__ cbox_out,
                             int32_t* __restrict__ child, float* __restrict__ ibox) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const uint64_t f = flags[i];
  if (!(f >> 32)) return;
  const uint64_t x = scanned[i] + sums[i / kScanTile];
  const uint32_t dst = uint32_t(x >> 32);
  float b[6];
  for (int k = 0; k < 6; ++k) b[k] = cbox[size_t(i) * 6 + k];
  int32_t ref = cref[i];
  if (f & 1ull) {
    const int j = nn[i];
    const int32_t id = next_id - int32_t(x & 0xFFFFFFFFull);
    child[2 * size_t(id)] = ref;
    child[2 * size_t(id) + 1] = cref[j];
    for (int k = 0; k < 3; ++k) {
      b[k] = fminf(b[k], cbox[size_t(j) * 6 + k]);
      b[3 + k] = fmaxf(b[3 + k], cbox[size_t(j) * 6 + 3 + k]);
    }
    for (int k = 0; k < 6; ++k) ibox[size_t(id) * 6 + k] = b[k];
    ref = id;
  }
  cref_out[dst] = ref;
  for (int k = 0; k < 6; ++k) cbox_out[size_t(dst) * 6 + k] = b[k];
}

__global__ void k_ploc_init(const float* __restrict__ leaf_box, uint32_t n, int32_t* __restrict__ cref,
                            float* __restrict__ cbox) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  cref[i] = ~int32_t(i);
  for (int k = 0; k < 6; ++k) cbox[size_t(i) * 6 + k] = leaf_box[size_t(i) * 6 + k];
}

__device__ __forceinline__ float wlo(float x, float s) { return __fsub_rn(x, __fmul_rn(__fadd_rn(fabsf(x), s), 0x1p-20f)); }
__device__ __forceinline__ float whi(float x, float s) { return __fadd_rn(x, __fmul_rn(__fadd_rn(fabsf(x), s), 0x1p-20f)); }

// Traversal layout (as k_pack_nodes): both children's boxes, widened by
// (|x| + scene scale) * 2^-20 so the box tests stay conservative, and refs.
__global__ void k_ploc_pack(const int32_t* __restrict__ child, const float* __restrict__ ibox,
                            const float* __restrict__ leaf_box, uint32_t n, float4* __restrict__ nodes) {
  const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id + 1 >= n) return;
  const float* r = ibox;  // root = node 0
  const float scale = fmaxf(fmaxf(fmaxf(fabsf(r[0]), fabsf(r[1])), fmaxf(fabsf(r[2]), fabsf(r[3]))),
                            fmaxf(fabsf(r[4]), fabsf(r[5])));
  const int32_t c0 = child[2 * size_t(id)], c1 = child[2 * size_t(id) + 1];
  const float* p0 = c0 >= 0 ? ibox + 6 * size_t(c0) : leaf_box + 6 * size_t(~c0);
  const float* p1 = c1 >= 0 ? ibox + 6 * size_t(c1) : leaf_box + 6 * size_t(~c1);
  float b0[6], b1[6];
  for (int a = 0; a < 3; ++a) {
    b0[a] = wlo(p0[a], scale); b0[3 + a] = whi(p0[3 + a], scale);
    b1[a] = wlo(p1[a], scale); b1[3 + a] = whi(p1[3 + a], scale);
  }
  pack_node(nodes + 4 * size_t(id), b0, b1, c0, c1);
}

namespace {
struct PlocScratch {
  int32_t* cref[2];
  float* cbox[2];
  int32_t* nn;
  uint64_t* flags;
  uint64_t* scanned;
  uint64_t* sums;
  uint64_t* total;
  int32_t* child;
  float* ibox;
};
size_t carve(uint32_t n, char* base, PlocScratch* s) {
  size_t off = 0;
  auto take = [&](size_t bytes) { char* p = base ? base + off : nullptr; off += (bytes + 255) & ~size_t(255); return p; };
  const uint32_t nb = (n + kScanTile - 1) / kScanTile + 1;
  for (int k = 0; k < 2; ++k) {
    s->cref[k] = reinterpret_cast<int32_t*>(take(size_t(n) * 4));
    s->cbox[k] = reinterpret_cast<float*>(take(size_t(n) * 24));
  }
  s->nn = reinterpret_cast<int32_t*>(take(size_t(n) * 4));
  s->flags = reinterpret_cast<uint64_t*>(take(size_t(n) * 8));
  s->scanned = reinterpret_cast<uint64_t*>(take(size_t(n) * 8));
  s->sums = reinterpret_cast<uint64_t*>(take(size_t(nb) * 8));
  s->total = reinterpret_cast<uint64_t*>(take(8));
  s->child = reinterpret_cast<int32_t*>(take(size_t(2) * n * 4));
  s->ibox = reinterpret_cast<float*>(take(size_t(n) * 24));
  return off;
}
}  // namespace

size_t ploc_scratch_bytes(uint32_t ntris) {
  PlocScratch s;
  return carve(ntris, nullptr, &s);
}

int launch_ploc_build(const float* leaf_box, uint32_t n, float4* nodes, void* scratch, cudaStream_t st,
                      int* launches) {
  if (n < 2) return 0;
  PlocScratch s;
  carve(n, static_cast<char*>(scratch), &s);
  int L = 0, cur = 0;
  k_ploc_init<<<(n + 255) / 256, 256, 0, st>>>(leaf_box, n, s.cref[0], s.cbox[0]); ++L;
  uint32_t m = n;
  int32_t next_id = int32_t(n) - 2;
  int max_rounds = 64;
  for (uint32_t x = n; x > 1; x >>= 1) max_rounds += 8;
  for (int round = 0; m > 1; ++round) {
    if (round > max_rounds) return 1;  // stalled (degenerate input): the caller keeps the LBVH tree
    const uint32_t g = (m + kPlocT - 1) / kPlocT, nb = (m + kScanTile - 1) / kScanTile;
    k_ploc_nn<<<g, kPlocT, 0, st>>>(s.cbox[cur], m, s.nn);
    k_ploc_flags<<<(m + 255) / 256, 256, 0, st>>>(s.nn, m, s.flags);
    k_scan_tiles<<<nb, kScanT, 0, st>>>(s.flags, m, s.scanned, s.sums);
    k_scan_sums<<<1, 1024, 0, st>>>(s.sums, nb, s.total);
    k_ploc_merge<<<(m + 255) / 256, 256, 0, st>>>(s.cref[cur], s.cbox[cur], s.nn, s.flags, s.scanned, s.sums, m,
                                                   next_id, s.cref[cur ^ 1], s.cbox[cur ^ 1], s.child, s.ibox);
    L += 5;
    uint64_t tot = 0;
    if (cudaMemcpyAsync(&tot, s.total, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return -1;
    const uint32_t made = uint32_t(tot & 0xFFFFFFFFull), kept = uint32_t(tot >> 32);
    if (made == 0 || kept + made != m) return -1;
    next_id -= int32_t(made);
    m = kept;
    cur ^= 1;
  }
  if (next_id != -1) return -1;
  k_ploc_pack<<<(n - 1 + 255) / 256, 256, 0, st>>>(s.child, s.ibox, leaf_box, n, nodes); ++L;
  if (launches) *launches += L;
  return 0;
}

}  // namespace vlbk
