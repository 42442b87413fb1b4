// vlb_internal.h -- host-side structures and kernel launchers shared by the
// C ABI (vlb_api.cpp) and the CUDA translation units.  Not installed.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/vlb.h"

namespace vlbk {

// Device error counters (one int each) kept per context.
enum ErrSlot : int {
  kErrStackOverflow = 0,  // BVH traversal stack overflow
  kErrTimeout = 1,        // bounded mbarrier / flag wait gave up
  kErrBadInput = 2,       // device-side argument check
  kErrBounds = 3,         // bounds-check build: an index outside its array
  kErrSlots = 8
};

// Bounds-check build (compiled with -DVLB_BOUNDS_CHECK): VLB_INB(i, n, err) is
// false for an index outside [0, n) and counts it in err[kErrBounds]; the
// caller then skips the access or ends the walk.  VLB_CLAMP(i, n, err) maps
// such an index to 0 (for reads whose value only feeds arithmetic).  In the
// normal build they are `true` and `i`: no code.
#if defined(VLB_BOUNDS_CHECK) && defined(__CUDACC__)
__device__ __forceinline__ bool inb_checked(long long i, long long n, int* err) {
  if (i >= 0 && i < n) return true;
  if (err) atomicAdd(err + kErrBounds, 1);
  return false;
}
#define VLB_INB(i, n, err) (::vlbk::inb_checked((long long)(i), (long long)(n), (err)))
#define VLB_CLAMP(i, n, err) (VLB_INB(i, n, err) ? (i) : 0)
#else
#define VLB_INB(i, n, err) true
#define VLB_CLAMP(i, n, err) (i)
#endif

// Sizes of the bake's trace kernels: the warp stack of the packet walk and
// the per-lane stacks of the lane walks (a wide node pushes up to 7 children).
constexpr int kTraceStack = 64;
constexpr int kLaneStack = 96;

// ---- binary traversal node (64 bytes) -------------------------------------------
// The two children's boxes (lo xyz, hi xyz) grouped by axis, so that one
// packed FMA (fma.rn.f32x2) takes one child's x and y planes, or its two z
// planes, at once, then the children's references (>= 0 a node slot, < 0 the
// complement of a triangle slot):
//   [lx0 ly0 hx0 hy0] [lx1 ly1 hx1 hy1] [lz0 hz0 lz1 hz1] [ref0 ref1 0 0]
#ifdef __CUDACC__
#define VLB_HD __host__ __device__
#else
#define VLB_HD
#endif
VLB_HD inline float ref_bits(int32_t r) {
  float f;
  std::memcpy(&f, &r, 4);
  return f;
}
VLB_HD inline void pack_node(float4* q, const float* b0, const float* b1, int32_t c0, int32_t c1) {
  q[0] = make_float4(b0[0], b0[1], b0[3], b0[4]);
  q[1] = make_float4(b1[0], b1[1], b1[3], b1[4]);
  q[2] = make_float4(b0[2], b0[5], b1[2], b1[5]);
  q[3] = make_float4(ref_bits(c0), ref_bits(c1), 0.f, 0.f);
}
inline void unpack_node(const float4* q, float* b0, float* b1, int32_t* c0, int32_t* c1) {
  const float x0[6] = {q[0].x, q[0].y, q[2].x, q[0].z, q[0].w, q[2].y};
  const float x1[6] = {q[1].x, q[1].y, q[2].z, q[1].z, q[1].w, q[2].w};
  std::memcpy(b0, x0, sizeof x0);
  std::memcpy(b1, x1, sizeof x1);
  std::memcpy(c0, &q[3].x, 4);
  std::memcpy(c1, &q[3].y, 4);
}

// ---- skybox projection ------------------------------------------------------
struct SkyboxArgs {
  const void* texels;     // device, count maps back to back
  int fmt;                // vlb_texel_format
  int layout;             // vlb_sky_layout
  uint32_t w, h;          // cubemap: w == h == face size
  uint32_t count;         // maps
  uint32_t lmax;          // 2 or 3
  uint32_t flags;         // VLB_SKY_REF_BGRA_SWAP
  uint32_t texels_per_map;
  uint32_t slab_texels;   // texels per work unit (multiple of the chunk)
  uint32_t slabs_per_map;
  uint32_t group;         // maps per work unit (1, 2 or 4)
  const float* solid_angle;  // cubemap: w*w table (same for every face)
  const float2* pair_table;  // cubemap, optional: launch_cube_pair_table's layout (selects the group kernel)
  const float2* col_tab;     // panorama: w entries (cos phi, sin phi)
  const float4* row_tab;     // panorama: h entries (sin theta, cos theta, weight, 0)
  float* partial;            // count*slabs_per_map*K*3
  int* err;
  uint32_t hold_producer;    // test hook: the producer warp issues nothing
  uint32_t wait_polls;       // bounded-wait polls (0: kWaitPolls)
};
// The skybox kernel writes one partial per (map, slab, consumer warp):
// partial[map][slab][warp][v], kSkyPartialsPerSlab warps.
constexpr int kSkyPartialsPerSlab = 8;
void launch_cube_solid_angle(float* out, uint32_t n, cudaStream_t s);
// Weighted basis of texel pairs per 256-texel chunk, [chunk][k][128] float2
// (FP64, rounded once), for the group kernel of cubemap batches.
size_t cube_pair_table_bytes(uint32_t n, uint32_t lmax);
void launch_cube_pair_table(float2* out, uint32_t n, uint32_t lmax, cudaStream_t s);
// Fills slab_texels / slabs_per_map / group from texels_per_map, count and
// lmax.  The slab is 8192 texels whatever the batch (so a map's sums have one
// order); max_slabs > 0 caps the slabs per map by widening the slab.
void skybox_plan(SkyboxArgs& a, uint32_t max_slabs);
// Returns the partials per map it wrote (the slab count for launch_sh_finalize).
int launch_skybox_sh(const SkyboxArgs& a, bool tma, int num_sms, cudaStream_t s);
// out[m][v] = sum_j partial[m][j][v] in FP64, j in fixed order.
void launch_sh_finalize(const float* partial, uint32_t nmaps, uint32_t slabs, uint32_t nvals, float* out,
                        cudaStream_t s);

// ---- projection of a radiance tile --------------------------------------------
// `partial`: project_partial_bytes(nprobes, S, K) of device scratch (null when
// that is 0: the tile is projected unsplit).
size_t project_partial_bytes(uint32_t nprobes, uint32_t S, uint32_t K);
void launch_project_f32(const float* radiance, uint32_t nprobes, uint32_t S, const float* basis16, uint32_t K,
                        float* out, float* partial, cudaStream_t s, int* err = nullptr, int num_sms = 0,
                        uint32_t hold = 0, uint32_t wait_polls = 0);
// The TMA-staged form of the unsplit FP32 projection (same bits); returns 0
// when the tile does not qualify (S % 4, alignment) and nothing was launched.
int launch_project_f32_tma(const float* radiance, uint32_t nprobes, uint32_t S, const float* basis16, uint32_t K,
                           float* out, int* err, int num_sms, cudaStream_t s, uint32_t hold, uint32_t wait_polls);
// split: the tile is [rows][2S] hi/lo BF16 pairs (the sample is hi + lo).
void launch_project_bf16_simt(const uint16_t* radiance, uint32_t nprobes, uint32_t S, const float* basis16,
                              uint32_t K, float* out, float* partial, uint32_t split, cudaStream_t s);
// tcgen05 projection of a BF16 tile (k_project_tc.cu).  basis_bt: [32][bt_pitch]
// BF16, rows 0..15 the high and 16..31 the low part of the weighted basis.
// Needs S % 8 == 0 and a 16-byte aligned tile; returns -1 if the tensor maps
// cannot be built.
bool project_tc_supported(const void* radiance, uint32_t S);
// hold / wait_polls: vlb_ctx_test_hook (0, 0 in normal use).
int launch_project_tc(const uint16_t* radiance, uint32_t nprobes, uint32_t S, const uint16_t* basis_bt,
                      uint32_t bt_pitch, uint32_t K, float* out, int* err, int num_sms, cudaStream_t s,
                      uint32_t hold = 0, uint32_t wait_polls = 0);
// out[p][v] <- sum over q <= p of out[q][v] (FP64 running sum, one rounding).
void launch_probe_prefix(float* out, uint32_t nprobes, uint32_t V, cudaStream_t s);
void launch_sh_eval_envmap(const float* coeffs, uint32_t K, uint32_t w, uint32_t h, float scale, const float2* col_tab,
                           const float4* row_tab, float* out, cudaStream_t s);

// ---- LBVH ---------------------------------------------------------------------
struct LbvhBuild {
  // inputs
  const float* positions;  // device
  uint32_t stride_floats;
  uint32_t nverts;
  const uint32_t* indices;  // device
  const float* albedo;      // device ntris*3 or null
  uint32_t ntris;
  // outputs (device, allocated by the caller)
  uint32_t* codes;   // n sorted
  uint32_t* order;   // n sorted -> original
  int32_t* child;    // 2(n-1)
  float* box;        // (2n-1)*6
  float4* nodes;     // (n-1)*4
  float4* tris;      // n*3 (sorted order): v0|id, e1, e2
  float4* tri_albedo;  // n (by original index)
  // scratch (device)
  void* scratch;
  size_t scratch_bytes;
};
size_t lbvh_scratch_bytes(uint32_t ntris);
void launch_lbvh_build(const LbvhBuild& b, cudaStream_t s, int* launches);
// Traversal tree by PLOC clustering over the Morton-sorted leaves
// (k_ploc.cu): overwrites `nodes` (root 0) and returns 0; returns 1 with
// `nodes` untouched if clustering stalls (more than 64 + 8 log2 n rounds),
// -1 on a CUDA error or a round that merges nothing.
size_t ploc_scratch_bytes(uint32_t ntris);
int launch_ploc_build(const float* leaf_box, uint32_t n, float4* nodes, void* scratch, cudaStream_t s,
                      int* launches);
// Permutation of the probes by 24-bit Morton code inside `bounds` (min xyz,
// max xyz), so that each 32-probe packet is spatially compact; also zeroes
// *zero_word (the trace's work counter; may be null) in stream order.
// Returns the number of kernels launched.
size_t probe_order_scratch_bytes(uint32_t n);
int launch_probe_order(const float* probes, uint32_t n, const float bounds[6], uint32_t* order, void* scratch,
                       uint32_t* zero_word, cudaStream_t s);

// ---- trace + shade --------------------------------------------------------------
struct TraceArgs {
  const float4* nodes;
  const float4* wnodes;   // 8-wide quantised tree: the lane walks use it when set (same results)
  const float4* tris;
  const float4* albedo;
  uint32_t ntris;
  uint32_t nwide;         // wide nodes
  const float* probes;    // device nprobes*3
  const uint32_t* order;  // device permutation: packet slot -> probe index
  uint32_t nprobes;
  const float4* dirs;     // device S (xyz), caller order
  const float4* dinv;     // device S: per-axis reciprocals of dirs (zero components nudged to 1e-30)
  const uint32_t* dir_order;  // device S: trace position -> direction index (grouped by octant)
  uint32_t S;
  float3 sun;             // unit
  float3 sun_inv;         // per-axis reciprocals of sun, as dinv
  float sun_scale;        // intensity / pi
  float tmin, tmax, bias;
  const float* sky;       // device cubemap or null
  uint32_t sky_n;
  uint32_t shading;       // vlb_shading
  float3 light;           // VLB_SHADE_REF_PHONG point light
  // outputs
  float* radiance;        // [nprobes][3][S] fp32 or null
  uint16_t* radiance_bf16;  // [nprobes][3][S] bf16, or [nprobes][3][2S] hi/lo split, or null
  uint32_t bf16_split;    // 1: radiance_bf16 holds hi/lo pairs (store_bf16)
  int32_t* hit_tri;       // [nprobes*S] or null
  uint8_t* shadow;        // [nprobes*S] or null
  float* dbg_radiance;    // [nprobes*S*3] or null
  // fused projection
  const float* basis16;   // S x 16 fp32 weighted basis
  uint32_t K;
  float* partial;         // [nprobes][block chunks][K*3]
  uint32_t* group_done;   // [probe groups] completion counters (zero before the launch)
  uint32_t* work_counter; // next (packet, CTA chunk) item for the persistent CTAs (zero before the launch)
  float* out;             // [nprobes][K][3]
  // decomposition: a work item is one 32-probe packet and one chunk of
  // dirs_per_warp consecutive directions; persistent warps pull items
  uint32_t dirs_per_warp;
  uint32_t chunks;        // direction chunks per packet
  uint32_t lane;          // 1: per-lane traversal, 0: packet traversal
  uint32_t ray_block;     // tile lane walk: rays a warp takes from the counter at once (set by its launch)
  unsigned long long* counters;  // null, or [warp node fetches, warp triangle fetches, shadow rays, lane node tests]
  int* err;
  // grid mode (null grid_hdr: tree walks): grid g < S for direction g, grid S for the sun
  float4* grid_hdr;       // [S+1][4]: (u, lo_u), (v, lo_v), (d / |d|^2, 1 / cell_u), (1 / cell_v, ok, -, -)
  uint32_t* grid_cells;   // [S+1][G*G+1] entry offsets per cell
  uint16_t* grid_ent;     // [S+1][kGridCap] triangle slots, cell by cell, by near depth
  float4* grid_box;       // [S+1][ntris] widened 2D boxes (umin, umax, vmin, vmax)
  float2* grid_dep;       // [S+1][ntris] depth range along d in units of t
  uint32_t grid_g;        // cells per side
  float grid_margin;      // 2^-12 of the scene's coordinate scale
  float grid_far;         // origins with a larger coordinate walk the tree
};
constexpr int kGridThreads = 256;
constexpr uint32_t kGridMaxTris = 4096;  // grid mode's triangle limit
constexpr uint32_t kGridCap = 24576;     // entries per grid
size_t grid_build_smem(uint32_t G, uint32_t ntris);
bool grid_supported(uint32_t ntris, uint32_t nprobes, uint32_t S);
void launch_grid_build(const TraceArgs& a, cudaStream_t s);
constexpr int kTraceWarps = 4;
// 1/d with zero components nudged to +-1e-30, the reciprocal every ray setup
// uses: one IEEE FP32 division, so host and device give the same bits.
inline float host_safe_inv(float d) { return 1.0f / (std::fabs(d) > 1e-30f ? d : std::copysign(1e-30f, d)); }
// Chooses dirs_per_warp / chunks for nprobes x S rays on num_sms SMs: fine
// items for load balance, coarser in fused mode where each item leaves a
// K x 3 partial per probe.
void plan_trace(TraceArgs& a, int num_sms, bool fused);
// Persistent launches: at most num_sms x (resident CTAs per SM) CTAs pull
// items from a.work_counter, which must be zero before the launch.
void launch_trace_tile(const TraceArgs& a, int num_sms, cudaStream_t s);
void launch_trace_fused(const TraceArgs& a, int num_sms, cudaStream_t s);

// ---- batched bakes: many jobs (scene, probes, direction set) in one launch -------
struct BakeJobDev {
  // scene and shading (the fields trace_sample reads)
  const float4* nodes;
  const float4* wnodes;   // 8-wide quantised tree or null
  const float4* tris;
  const float4* albedo;
  uint32_t ntris;
  uint32_t nwide;         // wide nodes
  float tmin, tmax, bias;
  float3 sun;
  float3 sun_inv;
  float sun_scale;
  const float* sky;
  uint32_t sky_n;
  uint32_t shading;       // vlb_shading
  float3 light;           // VLB_SHADE_REF_PHONG point light
  int* err;
  // probes and directions
  const float* probes;    // device nprobes*3
  uint32_t* order;        // device nprobes: packet slot -> probe (written by the batched sort)
  uint32_t nprobes;
  const float4* dirs;
  const float4* dinv;
  const uint32_t* dir_order;
  uint32_t S;
  // this job's rows of its direction set's radiance tile
  float* radiance;
  uint16_t* radiance_bf16;
  uint32_t bf16_split;    // 1: hi/lo pairs, rows of 2S
  // rays [ray_begin, ray_begin + P * S) of the batch's numbering (P: nprobes
  // rounded up to 32), the range rounded up to whole chunks
  uint32_t ray_begin;
  // probe sort: bounds for the Morton codes, 4 scratch arrays of nprobes
  float bounds[6];
  uint32_t* sort_scratch;
  // kept primary hits, [nprobes][S] (triangle slot or -1, distance bits):
  // written when hits_out is set; when hits_in is set the primary walk is
  // skipped and the kept hit shaded (relight)
  int2* hits_out;
  const int2* hits_in;
  // fused projection (no radiance tile): a work item is one probe and one
  // chunk of chunk_rays consecutive positions of the trace order
  const float* basis16;   // S x 16 FP32 weighted basis
  float* out;             // [nprobes][K][3], this job's rows
  float* partial;         // [nprobes][chunks][K*3] FP32 chunk sums (chunks > 1)
  uint32_t* done;         // [nprobes] chunk tickets, zero before the launch
  uint32_t chunks, chunk_rays;
  // item order: 0 probe-major (a probe's chunks in a row: the rays in flight
  // share origins), 1 chunk-major (every probe's chunk c in a row: the basis
  // rows of chunk c are read once from HBM while all probes use them; for
  // direction sets whose basis does not stay in L2).  Results do not depend on it.
  uint32_t chunk_major;
  uint32_t item_begin;    // first work item of this job in the launch's numbering
  // per-ray debug outputs of the fused walk (null: none), ray r = probe * S + s
  int32_t* hit_tri;
  uint8_t* shadow;
  float* dbg_radiance;
};
// Fused lane walk: chunk size for S directions, a multiple of 64 rays, at
// most 4 chunks per probe while a chunk holds at most 4096 rays (larger sets,
// such as the 3141 x 1000 equirect set, get more chunks).  Large chunks keep
// a warp on one probe's neighbouring directions for longer, so its rays reuse
// the nodes it just fetched (4 chunks of 256 rays on the 64^3-probe, 1024-direction bake:
// 9.5 % faster than 16 of 64).  A function of S alone, so a probe's sums have
// the same order in a single bake and in any batch.
constexpr uint32_t kFusedSubRays = 64;
constexpr uint32_t kFusedMaxChunks = 4;
constexpr uint32_t kFusedMaxChunkRays = 4096;
inline uint32_t fused_chunk_rays(uint32_t S) {
  const uint32_t per = (S + kFusedMaxChunks - 1) / kFusedMaxChunks;
  const uint32_t d = (per + kFusedSubRays - 1) / kFusedSubRays * kFusedSubRays;
  return d < kFusedMaxChunkRays ? d : kFusedMaxChunkRays;
}
// Chunk-major item order when the direction set's basis (64 B a direction)
// exceeds 16 MiB.
inline uint32_t fused_chunk_major(uint32_t S) { return uint64_t(S) * 64 > (16ull << 20) ? 1u : 0u; }
// Launch knobs of the fused walk (vlb_batch_schedule; results do not depend on them).
struct FusedSched {
  uint32_t ctas_per_sm = 8;  // register budget: 7, 8 or 9 resident 4-warp CTAs per SM
  uint32_t node_steps = 6;   // inner-node steps per turn
  uint32_t refill_idle = 32; // idle lanes that trigger a refill
};
// One persistent launch: warps pull work items (job, probe, direction chunk)
// from *counter (zero before the launch), trace them per lane and project
// each chunk's radiance in the warp (FP32 sums in a fixed order, chunk sums
// added in FP64 in chunk order by the chunk that finishes last).  njobs == 1
// passes the job by value (jobs may be null).  The jobs share one shading,
// read from `one` (for a table, the host copy of its first job).
void launch_trace_fused_lane(const BakeJobDev* jobs, const BakeJobDev& one, uint32_t njobs, uint32_t total_items,
                             uint32_t K, uint32_t* counter, const FusedSched& sc, int num_sms, cudaStream_t s);
// One CTA per job: spatial order of each job's probes into job.order
// (counting sort on a 12-bit Morton prefix up to 16,384 probes, the CTA
// radix sort in the job's sort scratch above).
void launch_probe_order_batch(const BakeJobDev* jobs, uint32_t njobs, cudaStream_t s);
// Persistent trace over all jobs' rays (tile output), warps taking chunks of
// `chunk` rays (a multiple of 32); counter zeroed before.
// ref_shading: every job's shading is VLB_SHADE_REF_PHONG (else every job's is Lambert + sun).
void launch_trace_batch(const BakeJobDev* jobs, uint32_t njobs, uint32_t total_rays, uint32_t chunk,
                        uint32_t* counter, bool ref_shading, int num_sms, cudaStream_t s);
// Copies job j's rows of a projected group output to its own output:
// dst[j] <- src + src_row0[j]*K*3 floats, nprobes[j]*K*3 floats.
void launch_scatter_rows(const float* src, float* const* dst, const uint32_t* src_probe0, const uint32_t* nprobes,
                         uint32_t njobs, uint32_t K, cudaStream_t s);

// ---- probe evaluation (consumer side of the baked grid) ----------------------------
struct ProbeEvalArgs {
  const float4* nodes;
  const float4* tris;
  uint32_t ntris;           // 0: every probe visible
  const float* coeffs;      // nprobes x K x 3, the bake's breadth-first grid order
  float org[3], step[3];
  uint32_t counts[3];
  const float* points;      // n x 3
  const float* normals;     // n x 3 (normalised in the kernel)
  uint32_t n;
  float bias;
  float* out;               // n x 3
  uint8_t* vis;             // n, bit c = corner c visible (or null)
  int* err;
};
void launch_probe_eval(const ProbeEvalArgs& a, uint32_t lmax, cudaStream_t s);
// out[i] = sum_k c_k Y_k(normalize(dirs[i])), K = (lmax+1)^2 coefficients.
void launch_sh_eval_dirs(const float* coeffs, uint32_t lmax, const float* dirs, uint32_t n, float* out,
                         cudaStream_t s);
// RGBA8 UNORM from RGB floats: scale, optional sRGB, clamp, round; alpha 255.
void launch_encode_rgba8(const float* rgb, size_t n, float scale, uint32_t srgb, uint8_t* out, int num_sms,
                         cudaStream_t s);

}  // namespace vlbk

// ---- host internals shared by the C ABI translation units ----------------------
namespace vlbh {
// Per-job extras of a batch: kept primary hits out, or kept hits in (relight).
struct JobExt {
  int2* hits_out = nullptr;
  const int2* hits_in = nullptr;
};
vlb_status batch_launch(vlb_ctx* ctx, const vlb_bake_job* jobs, const JobExt* ext, uint32_t njobs,
                        const vlb_bake_params* params, const vlb_batch_schedule& sc, bool* host_out_any);
// Launch-error check, and (sync) stream synchronisation + device error counters.
vlb_status ctx_finish(vlb_ctx* ctx, bool sync);
// Collapses the scene's binary traversal tree into the 8-wide quantised tree
// (sc->wnodes, sc->nwide; wide_bvh.cpp).  Synchronous.
vlb_status build_wide(vlb_ctx* ctx, vlb_scene* sc);
// Re-lays the binary traversal tree with siblings in one 128-byte line
// (2n - 2 node slots); same tree, same results.
vlb_status pair_siblings(vlb_ctx* ctx, vlb_scene* sc);
vlb_status ctx_fail(vlb_ctx* ctx, vlb_status s, const char* msg);
}  // namespace vlbh

// ---- host objects behind the opaque handles ------------------------------------
struct vlb_ctx {
  int device = 0;
  vlb_ctx* parent = nullptr;  // a service's private context accepts its parent's objects
  int num_sms = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  int* d_err = nullptr;  // vlbk::kErrSlots ints
  int* h_err = nullptr;  // pinned host copy, read back with a synchronised call's last copy
  uint64_t launches = 0;
  bool host_inputs_pending = false;  // a host array was copied in by the current call
  bool profiling = false;
  struct Pending { std::string name; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  struct Stat { uint32_t launches = 0; double ms = 0; };
  std::map<std::string, Stat> stats;
  struct Buf { void* p = nullptr; size_t bytes = 0; };
  std::map<std::string, Buf> scratch;
  std::map<uint32_t, float*> cube_sa;  // solid-angle tables by face size
  std::map<uint64_t, float2*> cube_pt;  // texel-pair basis tables by (face size << 8 | lmax)
  // batched bakes: the shape key of the last batch, its captured graph (made
  // on the second call with that key) and the tuned schedule
  std::vector<uint64_t> batch_key;
  cudaGraphExec_t batch_exec = nullptr;
  uint32_t batch_graph_kernels = 0;
  std::vector<vlbk::BakeJobDev> batch_table;  // host copy of the job table
  std::vector<uint8_t> batch_meta;             // job table + scatter arrays, uploaded each call
  // vlb_batch_autotune's winners by scene-size class, and its last trials
  static constexpr int kSizeClasses = 4;
  vlb_batch_schedule tuned[kSizeClasses] = {};
  bool tuned_set[kSizeClasses] = {};
  std::vector<vlb_tune_trial> tune_log;
  uint32_t tune_class = 0;
  // vlb_ctx_test_hook: producers of the TMA pipelines issue nothing; waits
  // give up after wait_polls polls (0: the default bound)
  uint32_t hold_producer = 0, wait_polls = 0;
};

struct vlb_scene {
  vlb_ctx* ctx = nullptr;
  uint32_t ntris = 0, nverts = 0;
  float bounds[6] = {0, 0, 0, 0, 0, 0};
  uint32_t* codes = nullptr;
  uint32_t* order = nullptr;
  int32_t* child = nullptr;
  float* box = nullptr;
  float4* nodes = nullptr;
  float4* wnodes = nullptr;  // 8-wide quantised traversal tree (wide_bvh.cpp), or null
  uint32_t nwide = 0;
  float4* tris = nullptr;
  float4* albedo = nullptr;
  uint64_t bytes = 0;
};

struct vlb_dirset {
  vlb_ctx* ctx = nullptr;
  uint32_t n = 0;
  float4* d_dirs = nullptr;     // n trace directions
  float4* d_dinv = nullptr;     // n per-axis reciprocals of the trace directions (vlbk::host_safe_inv)
  uint32_t* d_order = nullptr;  // n direction indices sorted by ray octant (stable)
  uint16_t* d_bt = nullptr;     // [32][bt_pitch] BF16 weighted basis, high rows 0..15, low rows 16..31
  uint32_t bt_pitch = 0;
  // BF16 basis for hi/lo split tiles over 2S columns (built on first use):
  // rows 0..15 the high basis under both halves, rows 16..31 the low basis
  // under the high half and zero under the low half
  mutable std::mutex bt2_mu;
  mutable uint16_t* d_bt2 = nullptr;
  mutable uint32_t bt2_pitch = 0;
  float* d_basis16 = nullptr;   // n x 16 weighted basis, FP32
  std::vector<float> h_dirs;    // n*3
  std::vector<double> h_basis;  // n*16 FP64 weighted basis
  std::vector<float> h_basis32; // n*16
};

struct vlb_sky {
  vlb_ctx* ctx = nullptr;
  uint32_t n = 0;
  float* d_texels = nullptr;
};
