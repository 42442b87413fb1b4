// wide_bvh.cpp -- host passes over a scene's traversal tree: the 8-wide
// quantised tree (build_wide) and the sibling-pair node layout (pair_siblings).
//
// The binary traversal tree (PLOC clustering, or the LBVH) is collapsed into
// nodes of up to 8 children: starting from a binary node's two children, the
// internal child with the largest box surface area is replaced by its two
// children until there are 8 or no internal child is left (the greedy
// surface-area collapse of compressed wide BVHs, Ylitie, Karras and Laine,
// HPG 2017).  Each child keeps the box its binary parent stored for it (the
// widened traversal box), quantised to 8 bits per bound relative to the wide
// node: bound = fmaf(q, 2^e, origin) in FP32, one rounding.  Every bound is
// rounded outward and checked with that exact FP32 expression, so each
// quantised box contains the binary box it replaces.  The slab test is
// monotone in the box bounds, so a ray enters every wide box whose binary
// box it enters: the wide walk never prunes a triangle the binary walk keeps,
// and with the tie rule every ray's result is the binary walk's.
//
// Node layout (96 bytes, 6 x float4):
//   [0] origin x, y, z; w = bits: e_x | e_y << 8 | e_z << 16 | children << 24
//       (e: biased FP32 exponent of the axis scale 2^(e-127))
//   [1..3] twelve 32-bit words of bound bytes, children 0-3 then 4-7:
//       lo_x, hi_x, lo_y, hi_y, lo_z, hi_z of children 0-3 (byte c = child c),
//       then the same six words of children 4-7 (byte c = child 4 + c)
//   [4], [5] child references, int32: >= 0 a wide node, < 0 triangle slot ~r
// Children 0 .. count-1 are valid.  Node 0 is the root.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "vlb_internal.h"

namespace {

struct Child {
  int32_t ref;   // binary node (>= 0) or triangle slot (~slot)
  float box[6];  // lo xyz, hi xyz
};

float area(const float* b) {
  const float dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
  return dx * dy + dy * dz + dz * dx;
}

// The two children of binary node i (the 64-byte layout of vlbk::pack_node).
void binary_children(const float4* nodes, int32_t i, Child* c0, Child* c1) {
  vlbk::unpack_node(nodes + 4 * size_t(i), c0->box, c1->box, &c0->ref, &c1->ref);
}

// Quantises one axis of a wide node: scale 2^(e-127) and the bytes of each
// child's bounds, every bound rounded outward under the device's FP32
// dequantisation fmaf(q, scale, origin).
bool quantise_axis(const std::vector<Child>& kids, int a, float origin, uint32_t* e_out, uint8_t* qlo, uint8_t* qhi) {
  float top = origin;
  for (const Child& c : kids) top = std::max(top, c.box[3 + a]);
  const double ext = double(top) - double(origin);
  int e = 1;  // smallest normal scale 2^-126
  if (ext > 0.0) e = std::max(1, int(std::ceil(std::log2(ext / 255.0))) + 127);
  for (;; ++e) {
    if (e > 254) return false;
    const float s = std::ldexp(1.0f, e - 127);
    if (std::fmaf(255.f, s, origin) < top) continue;
    bool ok = true;
    for (size_t c = 0; c < kids.size() && ok; ++c) {
      const float lo = kids[c].box[a], hi = kids[c].box[3 + a];
      double ql = std::floor((double(lo) - double(origin)) / double(s));
      double qh = std::ceil((double(hi) - double(origin)) / double(s));
      int il = int(std::min(255.0, std::max(0.0, ql)));
      int ih = int(std::min(255.0, std::max(0.0, qh)));
      while (il > 0 && std::fmaf(float(il), s, origin) > lo) --il;
      while (ih < 255 && std::fmaf(float(ih), s, origin) < hi) ++ih;
      if (std::fmaf(float(il), s, origin) > lo || std::fmaf(float(ih), s, origin) < hi) ok = false;
      qlo[c] = uint8_t(il);
      qhi[c] = uint8_t(ih);
    }
    if (ok) break;
  }
  *e_out = uint32_t(e);
  return true;
}

}  // namespace

vlb_status vlbh::build_wide(vlb_ctx* ctx, vlb_scene* sc) {
  const uint32_t n = sc->ntris;
  if (n < 2) return VLB_OK;  // a walk of one triangle starts at the triangle
  std::vector<float4> bin(size_t(n - 1) * 4);
  if (cudaMemcpy(bin.data(), sc->nodes, bin.size() * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    return ctx_fail(ctx, VLB_ERR_CUDA, "wide tree: traversal tree download failed");
  }
  // breadth-first: queue of binary nodes that become wide nodes
  std::vector<int32_t> queue{0};
  std::vector<float4> wide;
  wide.reserve(size_t(n / 3 + 8) * 6);
  for (size_t qi = 0; qi < queue.size(); ++qi) {
    std::vector<Child> kids(2);
    binary_children(bin.data(), queue[qi], &kids[0], &kids[1]);
    while (kids.size() < 8) {
      int best = -1;
      float best_area = -1.f;
      for (size_t c = 0; c < kids.size(); ++c)
        if (kids[c].ref >= 0 && area(kids[c].box) > best_area) { best_area = area(kids[c].box); best = int(c); }
      if (best < 0) break;
      Child a, b;
      binary_children(bin.data(), kids[best].ref, &a, &b);
      kids[best] = a;
      kids.push_back(b);
    }
    float origin[3];
    for (int a = 0; a < 3; ++a) {
      origin[a] = kids[0].box[a];
      for (const Child& c : kids) origin[a] = std::min(origin[a], c.box[a]);
    }
    uint8_t q[3][2][8] = {};
    uint32_t e[3];
    for (int a = 0; a < 3; ++a)
      if (!quantise_axis(kids, a, origin[a], &e[a], q[a][0], q[a][1]))
        return ctx_fail(ctx, VLB_ERR_INTERNAL, "wide tree: a box could not be quantised");
    int32_t refs[8] = {};
    for (size_t c = 0; c < kids.size(); ++c) {
      if (kids[c].ref >= 0) {
        refs[c] = int32_t(queue.size());  // wide index of that child, in queue order
        queue.push_back(kids[c].ref);
      } else {
        refs[c] = kids[c].ref;
      }
    }
    float4 f[6];
    const uint32_t meta = e[0] | (e[1] << 8) | (e[2] << 16) | (uint32_t(kids.size()) << 24);
    f[0] = make_float4(origin[0], origin[1], origin[2], 0.f);
    std::memcpy(&f[0].w, &meta, 4);
    uint32_t words[12];
    for (int half = 0; half < 2; ++half)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 2; ++b) {
          uint32_t v = 0;
          for (int c = 0; c < 4; ++c) v |= uint32_t(q[a][b][4 * half + c]) << (8 * c);
          words[6 * half + 2 * a + b] = v;
        }
    std::memcpy(&f[1], words, 48);
    std::memcpy(&f[4], refs, 32);
    for (const float4& v : f) wide.push_back(v);
  }
  float4* dev = nullptr;
  if (cudaMalloc(&dev, wide.size() * sizeof(float4)) != cudaSuccess) {
    cudaGetLastError();
    return ctx_fail(ctx, VLB_ERR_OOM, "wide tree allocation failed");
  }
  if (cudaMemcpy(dev, wide.data(), wide.size() * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(dev);
    return ctx_fail(ctx, VLB_ERR_CUDA, "wide tree upload failed");
  }
  sc->wnodes = dev;
  sc->nwide = uint32_t(wide.size() / 6);
  sc->bytes += wide.size() * sizeof(float4);
  return VLB_OK;
}

// Sibling-pair layout of the binary traversal tree.  A walk that leaves node N
// goes to one of N's two children, and the lanes of a warp that leave N
// together go to either: storing both children in one 128-byte line (slots 2k
// and 2k + 1 of the 64-byte nodes) lets those lanes' fetches share a line.
// Slots are handed out depth first from the root (slot 0; slot 1 stays
// empty), a pair per node with an internal child (a half-empty pair when only
// one child is internal), so the array has at most 2n - 2 slots; it is
// allocated with exactly 2n - 2 (unused slots zero) so every slot index a walk
// can meet is inside it.  Only the storage changes: every walk visits the same
// nodes in the same order and returns the same bits.
vlb_status vlbh::pair_siblings(vlb_ctx* ctx, vlb_scene* sc) {
  const uint32_t n = sc->ntris;
  if (n < 3) return VLB_OK;  // one node: nothing to pair
  const size_t nold = n - 1, nslots = 2 * size_t(n) - 2;
  std::vector<float4> old(nold * 4);
  if (cudaMemcpy(old.data(), sc->nodes, old.size() * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    return ctx_fail(ctx, VLB_ERR_CUDA, "node layout: traversal tree download failed");
  }
  std::vector<float4> out(nslots * 4, make_float4(0.f, 0.f, 0.f, 0.f));
  // (old index, new slot) of nodes whose children still need slots
  std::vector<std::pair<int32_t, uint32_t>> stack{{0, 0}};
  uint32_t next = 2;
  while (!stack.empty()) {
    const auto [oi, ns] = stack.back();
    stack.pop_back();
    float4 q[4];
    for (int k = 0; k < 4; ++k) q[k] = old[4 * size_t(oi) + k];
    int32_t c[2];
    std::memcpy(&c[0], &q[3].x, 4);
    std::memcpy(&c[1], &q[3].y, 4);
    if (c[0] >= 0 || c[1] >= 0) {
      if (next + 2 > nslots) return ctx_fail(ctx, VLB_ERR_INTERNAL, "node layout: slot count exceeded");
      const uint32_t base = next;
      next += 2;
      uint32_t used = 0;
      int32_t nc[2] = {c[0], c[1]};
      for (int h = 0; h < 2; ++h)
        if (c[h] >= 0) {
          if (uint32_t(c[h]) >= nold) return ctx_fail(ctx, VLB_ERR_INTERNAL, "node layout: bad child");
          nc[h] = int32_t(base + used++);
        }
      std::memcpy(&q[3].x, &nc[0], 4);
      std::memcpy(&q[3].y, &nc[1], 4);
      // push the second child first so the first is laid out (and walked) first
      for (int h = 1; h >= 0; --h)
        if (c[h] >= 0) stack.push_back({c[h], uint32_t(nc[h])});
    }
    for (int k = 0; k < 4; ++k) out[4 * size_t(ns) + k] = q[k];
  }
  float4* dev = nullptr;
  if (cudaMalloc(&dev, out.size() * sizeof(float4)) != cudaSuccess) {
    cudaGetLastError();
    return ctx_fail(ctx, VLB_ERR_OOM, "node layout allocation failed");
  }
  if (cudaMemcpy(dev, out.data(), out.size() * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(dev);
    return ctx_fail(ctx, VLB_ERR_CUDA, "node layout upload failed");
  }
  cudaFree(sc->nodes);
  sc->nodes = dev;
  sc->bytes += nslots * 64 - nold * 64;
  return VLB_OK;
}
