/* vlb.h -- C ABI of the GB300 light-probe baker (libvlb.so).
 *
 * This is the drop-in boundary for the bake path of vulkan-light-bakery.
 * Plain pointers and sizes only; no C++ or torch types cross it.  Every
 * function returns a vlb_status; no exception leaves the library.  Each
 * declaration names the reference interface it replaces (paths inside the
 * reference project).
 *
 * Memory: every array argument may be host memory (pageable or pinned) or
 * device memory of the context's GPU; the library inspects each pointer.
 * A call whose arrays are all device pointers is asynchronous on the
 * context's stream: those arrays must stay valid until the stream passes the
 * call (vlb_ctx_synchronize, or an event the caller records on the stream).
 * A call with a host array returns after every host input has been read and
 * every host output written.  Nothing is retained beyond that.
 * A context is externally synchronised: one thread at a time, and calls on
 * one context run in stream order.
 */
#ifndef VLB_H
#define VLB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VLB_VERSION 1u

/* Replaces the reference's C++ exceptions (std::runtime_error, vk::SystemError,
 * caught in src/baker/main.cpp:26-40) and the printed-only fence failure of
 * src/application.cpp:265-273. */
typedef enum vlb_status {
  VLB_OK = 0,
  VLB_ERR_INVALID = 1,     /* bad argument (message in vlb_last_error) */
  VLB_ERR_OOM = 2,         /* device or host allocation failed */
  VLB_ERR_TIMEOUT = 3,     /* a bounded device wait gave up */
  VLB_ERR_CUDA = 4,        /* CUDA runtime error */
  VLB_ERR_UNSUPPORTED = 5, /* valid request this build does not implement */
  VLB_ERR_INTERNAL = 6     /* a device-side check fired (e.g. BVH stack overflow) */
} vlb_status;

typedef struct vlb_ctx vlb_ctx;
typedef struct vlb_scene vlb_scene;
typedef struct vlb_dirset vlb_dirset;
typedef struct vlb_sky vlb_sky;

/* ---- context ------------------------------------------------------------
 * Replaces Application::Application (src/application.cpp:540-556): device,
 * queues and command pools become one CUDA device + one stream. */
uint32_t vlb_version(void);
/* Build options of this library (no reference counterpart):
 * VLB_BUILD_BOUNDS_CHECK when compiled with -DVLB_BOUNDS_CHECK, the variant
 * whose kernels check every data-dependent index (tree nodes, triangle
 * slots, probe and direction permutations, sky texels, ring slots) and count
 * a violation (the call then returns VLB_ERR_INTERNAL) instead of using it. */
#define VLB_BUILD_BOUNDS_CHECK 1u
uint32_t vlb_build_flags(void);
const char* vlb_status_string(vlb_status s);
vlb_status vlb_ctx_create(int device, vlb_ctx** out);
/* Destroy every scene, direction set, sky and service made on a context
 * before the context itself: their destroy calls use it. */
void vlb_ctx_destroy(vlb_ctx* ctx);
/* Run the context's work on a caller-owned cudaStream_t (NULL restores the
 * context's own stream). */
vlb_status vlb_ctx_set_stream(vlb_ctx* ctx, void* cuda_stream);
void* vlb_ctx_get_stream(vlb_ctx* ctx);
vlb_status vlb_ctx_synchronize(vlb_ctx* ctx);
/* Message of the last failed call on this context (never NULL). */
const char* vlb_last_error(const vlb_ctx* ctx);

/* Per-kernel timing: when enabled, every kernel the library launches is
 * bracketed by CUDA events on the context's stream. */
typedef struct vlb_kernel_time {
  char name[48];
  uint32_t launches;
  double total_ms;
} vlb_kernel_time;
vlb_status vlb_ctx_set_profiling(vlb_ctx* ctx, int enable);
/* Synchronises, fills up to cap entries, returns the count in *n. */
vlb_status vlb_ctx_profile_read(vlb_ctx* ctx, vlb_kernel_time* out, uint32_t cap, uint32_t* n);
vlb_status vlb_ctx_profile_reset(vlb_ctx* ctx);
/* Kernels launched by the library on this context since creation. */
uint64_t vlb_ctx_launch_count(const vlb_ctx* ctx);
/* Test hook (no reference counterpart; the reference's only failure path is
 * an unbounded fence wait whose result is printed, src/application.cpp:
 * 265-273).  Makes the bounded device waits give up on purpose without
 * faulting the GPU: with VLB_HOOK_HOLD_PRODUCER the copy-issuing thread of
 * the TMA pipelines (the skybox projection's producer warp, the FP32 and the
 * tcgen05 projections' TMA threads) issues nothing, so no copy is ever in flight;
 * each waiting thread gives up after `wait_polls` mbarrier polls (0: the
 * library's bound), the kernel stops (the tcgen05 kernel frees its tensor
 * memory) and the call returns VLB_ERR_TIMEOUT.  hook 0 clears it; the
 * context stays usable and the next call succeeds. */
#define VLB_HOOK_HOLD_PRODUCER 1u
vlb_status vlb_ctx_test_hook(vlb_ctx* ctx, uint32_t hook, uint32_t wait_polls);

/* ---- probe grid -----------------------------------------------------------
 * Replaces LightBaker::probePositionsFromBoudingBox
 * (src/baker/light_baker.cpp:80-101): same FP32 arithmetic, same order (the
 * grid is grown one axis at a time: x runs first, then each existing probe is
 * repeated along y, then along z).  bounds = {min xyz, max xyz}; out_xyz
 * holds counts[0]*counts[1]*counts[2]*3 floats; grid_step may be NULL. */
vlb_status vlb_probe_grid_ref_order(const float bounds[6], const uint32_t counts[3], float* out_xyz,
                                    float grid_step[3]);

/* ---- scene ------------------------------------------------------------------
 * Replaces SceneManager::pushScene + Scene_t::buildAccelerationStructures
 * (src/scene_manager.cpp:1013-1034, :339-442): the hardware BLAS/TLAS becomes
 * a Morton LBVH built on the device (bit-exact with a CPU build).
 * positions: nverts vertices, position_stride_bytes apart (12 for packed xyz,
 * 48 for the reference's shader::Vertex, shaders/structures.h:20-26).
 * indices: ntris*3 u32.  tri_albedo: ntris*3 linear RGB, or NULL for 1. */
vlb_status vlb_scene_create(vlb_ctx* ctx, const float* positions, uint32_t position_stride_bytes, uint32_t nverts,
                            const uint32_t* indices, uint32_t ntris, const float* tri_albedo, vlb_scene** out);
/* The traversal tree is built by locally-ordered clustering (PLOC) of the
 * LBVH's Morton-sorted triangles (surface-area nearest neighbours): fewer
 * node visits per ray.  VLB_SCENE_TRAVERSAL_LBVH walks the Karras LBVH
 * itself instead.  Results do not depend on the tree; the exported BVH is
 * always the LBVH. */
#define VLB_SCENE_TRAVERSAL_LBVH 1u
/* Also build an 8-wide tree collapsed from the binary traversal tree, its
 * child boxes quantised to 8 bits per bound and rounded outward (96-byte
 * nodes), and walk it in the lane walks.  Results equal the binary walks' bit
 * for bit; it visits ~2.7x fewer nodes and fetches ~1.7x fewer bytes a ray,
 * but tests 8 boxes per node, and on the box scenes measured (778 to 786k
 * triangles) the extra box tests cost more than the saved fetches (the walk
 * is bound by instruction issue): opt-in. */
#define VLB_SCENE_TRAVERSAL_WIDE 2u
vlb_status vlb_scene_create_ex(vlb_ctx* ctx, const float* positions, uint32_t position_stride_bytes,
                               uint32_t nverts, const uint32_t* indices, uint32_t ntris, const float* tri_albedo,
                               uint32_t flags, vlb_scene** out);
void vlb_scene_destroy(vlb_scene* scene);
uint32_t vlb_scene_triangle_count(const vlb_scene* scene);
/* Replaces Scene_t::getBounds (src/scene_manager.cpp:214-217; the bounds are
 * grown in Scene_t::loadNode, :496-506).  The
 * reference starts its bounds at the origin, so include_origin=1 reproduces
 * it; 0 gives the plain vertex bounds. */
vlb_status vlb_scene_bounds(const vlb_scene* scene, int include_origin, float out[6]);
/* Copies the device LBVH to host arrays (any may be NULL): sorted Morton
 * codes [n], sorted triangle order [n], children [2(n-1)] (c >= 0 internal
 * node, c < 0 leaf ~c), boxes [(2n-1)*6] (internal nodes then leaves). */
vlb_status vlb_scene_bvh_export(const vlb_scene* scene, uint32_t* codes, uint32_t* order, int32_t* children,
                                float* boxes);
uint64_t vlb_scene_device_bytes(const vlb_scene* scene);

/* ---- sample direction sets -------------------------------------------------
 * A direction set is the rays every probe casts and the projection basis
 * that goes with them: trace direction d_s, basis direction b_s, weight w_s.
 * The projection is c_k = sum_s w_s Y_k(b_s) L(d_s). */
typedef enum vlb_frame {
  VLB_FRAME_WORLD = 0, /* basis evaluated at the traced direction */
  VLB_FRAME_XZY = 1    /* basis evaluated at the traced direction's .xzy */
} vlb_frame;
/* Spherical Fibonacci set of n directions, weight 4*pi/n. */
vlb_status vlb_dirset_create_fibonacci(vlb_ctx* ctx, uint32_t n, vlb_frame frame, vlb_dirset** out);
/* The reference's own sample set: one ray per w x h equirect pixel traced
 * along toVector(x2phi, y2theta).xzy (shaders/env_map.rgen:18-28) and
 * projected with the un-swizzled direction and weight (2pi/w)(pi/h)sin(theta)
 * (shaders/sh.comp:27-41).  Sample index s = y*w + x. */
vlb_status vlb_dirset_create_equirect(vlb_ctx* ctx, uint32_t w, uint32_t h, vlb_dirset** out);
/* Caller-defined set: n trace directions (xyz, unit length), optional basis
 * directions (NULL: the trace directions) and weights (FP64). */
vlb_status vlb_dirset_create(vlb_ctx* ctx, const float* trace_dirs, const float* basis_dirs, const double* weights,
                             uint32_t n, vlb_dirset** out);
void vlb_dirset_destroy(vlb_dirset* dirs);
uint32_t vlb_dirset_count(const vlb_dirset* dirs);
/* trace_dirs: n*3 FP32 as traced on the device; basis: n*16 FP32 weighted
 * basis values w_s*Y_k(b_s) (k = l(l+1)+m, l <= 3). Either may be NULL. */
vlb_status vlb_dirset_export(const vlb_dirset* dirs, float* trace_dirs, float* basis);

/* ---- skybox SH --------------------------------------------------------------
 * Replaces SkyboxManager::pushSkybox -> Skybox_t::computeSH
 * (src/skybox_manager.cpp:284-298, :107-130) and its shader
 * shaders/skybox_sh.comp.  Output: K x 3 FP32, K = (lmax+1)^2, coefficient
 * k = l(l+1)+m, RGB innermost (the reference's vec3 coeffs[16], scalar
 * layout).  lmax = 3 gives the reference's 16 coefficients. */
typedef enum vlb_sky_layout {
  VLB_SKY_CUBEMAP = 0,  /* 6 faces (+X,-X,+Y,-Y,+Z,-Z) of w x w texels, exact texel solid angles */
  VLB_SKY_PANORAMA = 1, /* w x h panorama, shaders/skybox_sh.comp:27-39 (phi - pi/2, basis at .xzy) */
  VLB_SKY_ENVMAP = 2    /* w x h equirect env map, shaders/sh.comp:27-39 */
} vlb_sky_layout;
typedef enum vlb_texel_format {
  VLB_TEXEL_RGB32F = 0, /* 3 floats per texel */
  VLB_TEXEL_RGBA8 = 1   /* 4 bytes per texel, UNORM (value/255), alpha ignored */
} vlb_texel_format;
/* flags: swap R and B, as the reference does by uploading RGBA bytes into a
 * B8G8R8A8 image (src/skybox_manager.cpp:18, src/application.cpp:690). */
#define VLB_SKY_REF_BGRA_SWAP 1u
vlb_status vlb_skybox_sh(vlb_ctx* ctx, const void* texels, vlb_texel_format fmt, vlb_sky_layout layout, uint32_t w,
                         uint32_t h, uint32_t lmax, uint32_t flags, float* out);
/* count maps stored back to back; out holds count*K*3 floats. */
vlb_status vlb_skybox_sh_batched(vlb_ctx* ctx, const void* texels, vlb_texel_format fmt, vlb_sky_layout layout,
                                 uint32_t w, uint32_t h, uint32_t count, uint32_t lmax, uint32_t flags, float* out);

/* No counterpart in the reference.  The same projection as vlb_skybox_sh
 * for callers that cannot allocate device memory when they call it (a
 * renderer whose device memory is all handed to its own pool, a host that
 * allows cudaMalloc only at start-up).  It takes no context and allocates
 * nothing: its scratch is a 557,312-byte __device__ array inside the
 * library, held by every GPU that loads the library until the process exits.
 * One map per call; lmax 2 or 3; cubemap faces up to 256, panoramas up to
 * 8192 x 8192; texels and out must be device memory of the current device
 * (host pointers, larger sizes and unknown flags return VLB_ERR_INVALID).
 * stream: a cudaStream_t or NULL; the call synchronises that stream and
 * returns when the result is in out.  The first call on a device looks up
 * the array's device address and keeps it, so make it before any stream
 * capture; calls after cudaDeviceReset are not supported (the array may
 * move).  All calls share the array: calls whose work overlaps on the GPU
 * race and must be serialised by the caller. */
vlb_status vlb_skybox_sh_noalloc(const void* texels, vlb_texel_format fmt, vlb_sky_layout layout, uint32_t w,
                                 uint32_t h, uint32_t lmax, uint32_t flags, float* out, void* stream);

/* Resident cubemap sky used on ray misses during a bake (the reference's
 * miss shader shaders/main.rmiss:37-41 reads an unbound set; this defines
 * it): nearest-texel lookup of a 6 x n x n RGB FP32 cubemap. */
vlb_status vlb_sky_create(vlb_ctx* ctx, const float* cubemap_rgb, uint32_t n, vlb_sky** out);
void vlb_sky_destroy(vlb_sky* sky);

/* ---- bake ---------------------------------------------------------------------
 * Replaces LightBaker::bake (src/baker/light_baker.cpp:287-328) with its
 * per-probe EnvMapGenerator::getMap (src/baker/env_map_generator.cpp:325-359:
 * env_map.rgen -> traversal -> env_map.rchit / shadow.rmiss / main.rmiss)
 * and dispatchBakingKernel (sh.comp).  probe_xyz: nprobes*3.  out: nprobes x
 * K x 3 FP32, probe-major, coefficient k = l(l+1)+m, RGB innermost; with
 * lmax = 3 this is byte-for-byte the reference's 192-byte-per-probe layout
 * (light_baker.cpp:294-322), each probe's own sum (the reference never clears
 * its accumulator between probes; that carry-over is not reproduced). */
typedef enum vlb_precision {
  VLB_PREC_FP32 = 0,  /* the default: FP32 radiance tile, FP32 projection (staged by TMA for large
                         tiles); the fastest path measured on the box scenes, within 1e-4 of FP64 */
  VLB_PREC_FUSED = 1, /* FP32, one kernel: each warp projects the rays it traced (FP32 sums in a
                         fixed order, FP64 chunk sums); no radiance tile */
  VLB_PREC_MIXED = 2, /* radiance stored as BF16 hi/lo pairs (4 bytes a sample), projected on the
                         tensor cores with the hi/lo BF16 basis and FP32 accumulation: within 1e-4
                         of FP64 like FP32 */
  VLB_PREC_BF16 = 3   /* radiance stored as one BF16 (2 bytes a sample), tensor-core projection with
                         the hi/lo basis: half the tile bytes, ~8 mantissa bits per sample (about
                         2e-3 relative SH error on lit box scenes) */
} vlb_precision;
/* vlb_bake_params.flags: with VLB_PREC_FUSED, always run the one-kernel packet
 * schedule (sun shading only: VLB_ERR_UNSUPPORTED with VLB_SHADE_REF_PHONG). */
#define VLB_BAKE_FORCE_FUSED_KERNEL 1u
/* vlb_bake_params.flags: traversal mode.  Packet: a warp walks the union of
 * its 32 probes' BVH paths once (coherent probes); lane: every ray walks its
 * own BVH path (probes sparse against the geometry); grid: the rays of each
 * direction are parallel, so each direction (and the sun) gets a 2D grid of
 * the projected triangles and a ray tests only its own cell (scenes of at
 * most 4096 triangles; others walk the tree; only on request).  Results do
 * not depend on the mode; without a bit every bake walks per lane (the
 * fastest on every scene measured). */
#define VLB_BAKE_TRAVERSAL_PACKET 2u
#define VLB_BAKE_TRAVERSAL_LANE 4u
#define VLB_BAKE_TRAVERSAL_GRID 8u

typedef struct vlb_bake_params {
  uint32_t lmax;          /* 2: 9 coefficients, 3: 16 (the reference) */
  uint32_t precision;     /* vlb_precision */
  uint32_t flags;         /* VLB_BAKE_* bits, normally 0 */
  float sun_dir[3];       /* direction toward the sun (normalised by the library) */
  float sun_intensity;    /* hit radiance = albedo * intensity/pi * max(0, n.l) * visibility */
  float tmin, tmax;       /* primary ray interval; shaders/env_map.rgen:22-23 use .001, 10000 */
  float shadow_bias;      /* shadow origin offset along the normal; shaders/env_map.rchit:81 uses .005 */
  const vlb_dirset* dirs; /* required */
  const vlb_sky* sky;     /* NULL: black sky */
  uint32_t shading;       /* vlb_shading */
  float light_pos[3];     /* VLB_SHADE_REF_PHONG: the point light (default 1, 10, 1: env_map.rchit:25) */
} vlb_bake_params;
/* vlb_bake_params.shading.
 * VLB_SHADE_LAMBERT_SUN (the benchmark configs): closest hit; the geometric
 * normal facing the ray; radiance = albedo * sun_intensity/pi * max(0, n.l) *
 * visibility of a shadow ray from hit + bias*n toward the sun; a miss takes
 * the sky cubemap (nearest texel) or black.
 * VLB_SHADE_REF_PHONG (the reference baker's own shading, replaces
 * shaders/env_map.rchit:51-102 with shaders/shadow.rmiss:6-9 and
 * shaders/main.rmiss:37-41): the normal of the triangle's winding (not turned
 * toward the ray; the reference interpolates the glTF vertex normals, which
 * equal it on flat-shaded geometry), L = normalize(light_pos - hit), a
 * shadow ray from hit + bias*n along L, any hit in (0, |light_pos - hit|),
 * traced only when n.L > 0; if it is not occluded, diffuse = 0.5 n.L and
 * specular = 0.5 max(0, reflect(L, n).d)^16 (ambient 0); the sample is
 * sRGB(albedo * (diffuse + specular)), and a miss sRGB(sky texel) or black
 * (the reference's bake binds no sky); every sample is then stored as
 * 8-bit UNORM (round(clamp(x, 0, 1) * 255) / 255) as the reference's
 * R8G8B8A8 env map (src/baker/env_map_generator.hpp:39) stores it, and the
 * projection reads the stored value.  The tile walks only (packet and grid
 * requests walk per lane). */
typedef enum vlb_shading { VLB_SHADE_LAMBERT_SUN = 0, VLB_SHADE_REF_PHONG = 1 } vlb_shading;
/* vlb_bake_params.flags: the reference's carry-over accumulator.  The
 * reference never clears its coefficient buffer between probes
 * (src/baker/light_baker.cpp:110-121, :298-322), so it writes for probe i
 * the sum of probes 0..i.  With this flag out[i] is that running sum, in the
 * order of probe_xyz, added in FP64 and rounded once (the reference's is a
 * racy FP32 sum); vlb_bake only (not batches or the service). */
#define VLB_BAKE_REF_ACCUMULATE 16u
void vlb_bake_params_default(vlb_bake_params* p);

/* Per-ray outputs for parity checks (any may be NULL; host or device):
 * ray r = probe*S + s.  hit_tri: original triangle index or -1.  shadow: 0
 * occluded, 1 lit, 2 no shadow ray (miss or n.l <= 0).  radiance: r*3 RGB. */
typedef struct vlb_bake_debug {
  int32_t* hit_tri;
  uint8_t* shadow;
  float* radiance;
} vlb_bake_debug;

vlb_status vlb_bake(vlb_ctx* ctx, const vlb_scene* scene, const float* probe_xyz, uint32_t nprobes,
                    const vlb_bake_params* params, float* out);
vlb_status vlb_bake_ex(vlb_ctx* ctx, const vlb_scene* scene, const float* probe_xyz, uint32_t nprobes,
                       const vlb_bake_params* params, float* out, const vlb_bake_debug* debug);
/* The asynchronous form of vlb_bake: probe_xyz and out must be device memory
 * of the context's GPU (VLB_ERR_INVALID otherwise).  The call enqueues the
 * bake on the context's stream and returns; done_event (a cudaEvent_t the
 * caller created, may be NULL) is recorded after the bake's last kernel.  The
 * arrays must stay valid until that event completes.  Device-side checks
 * (e.g. a traversal stack overflow) surface at the next synchronising call
 * on the context (vlb_ctx_synchronize). */
vlb_status vlb_bake_async(vlb_ctx* ctx, const vlb_scene* scene, const float* probe_xyz, uint32_t nprobes,
                          const vlb_bake_params* params, float* out, void* done_event);
/* Measurement aid (no reference counterpart; the reference's traversal is
 * inside the driver): one instrumented bake of the same rays, counting
 * out[0] primary rays, out[1] shadow rays, out[2] BVH node fetches (one per
 * 32-ray packet visit, or per lane in the lane walks), out[3] triangle
 * fetches (48 B each), out[4] node tests summed over rays, out[5] the bytes
 * of one node fetch (64 binary, 96 wide).  Host output. */
vlb_status vlb_bake_trace_stats(vlb_ctx* ctx, const vlb_scene* scene, const float* probe_xyz, uint32_t nprobes,
                                const vlb_bake_params* params, uint64_t out[6]);

/* ---- batched bakes ------------------------------------------------------------
 * No single reference counterpart: the reference bakes one scene per
 * LightBaker (src/baker/light_baker.cpp:20-74, src/baker/main.cpp:22-24) and one
 * probe per dispatch.  A batch bakes many (scene, probes) jobs at once: one
 * launch sorts every job's probes, ONE persistent trace launch has its warps
 * pull chunks of rays from all jobs (costliest jobs first) and hand them to
 * their lanes as the lanes free up, then one projection per direction set
 * writes all of that set's probes.  Each job's output is
 * bit-identical to vlb_bake of that job alone with the same parameters, in
 * every precision (VLB_PREC_FUSED: one persistent fused launch over all
 * jobs' work items, no tile and no projection launch).
 * The device part of a batch is captured in a CUDA graph on the second call
 * with the same shape (job count, per-job probe counts, direction sets,
 * output placement) and replayed while the shape repeats. */
typedef struct vlb_bake_job {
  const vlb_scene* scene;
  const float* probe_xyz;         /* nprobes*3, host or device */
  uint32_t nprobes;
  const vlb_bake_params* params;  /* NULL: the batch's; lmax and precision must equal the batch's */
  float* out;                     /* nprobes x K x 3, host or device */
} vlb_bake_job;
/* Schedule knobs of the batched trace (results do not depend on them). */
typedef struct vlb_batch_schedule {
  uint32_t dirs_per_item; /* tile walks: rays per lane in a warp's chunk of a job's rays (chunk = 32 x this),
                             1..64; 0 = library choice */
  uint32_t cost_order;    /* 1: work items of the costliest jobs (rays x log2 triangles) first */
  uint32_t graph;         /* 1: capture and replay the device part as a CUDA graph */
  uint32_t ctas_per_sm;   /* fused walk: resident 4-warp CTAs per SM its registers are sized for,
                             7, 8 or 9 (fewer: more registers a thread); 0 = 8 */
  uint32_t node_steps;    /* fused walk: inner-node steps of a lane turn before the leaf tests, 1..16;
                             0 = 6 */
  uint32_t refill_idle;   /* fused walk: idle lanes that make a warp hand out new rays, 1..32; 0 = 32 */
} vlb_batch_schedule;
/* sched NULL: the schedule vlb_batch_autotune stored in the context for the
 * batch's scene-size class (its largest scene: under 4,096, 65,536, 1,048,576
 * triangles, or more), else the library default {0, 1, 1, 0, 0, 0}.  A
 * VLB_PREC_FUSED vlb_bake uses the fused-walk knobs tuned for its scene's
 * class too. */
vlb_status vlb_bake_batch(vlb_ctx* ctx, const vlb_bake_job* jobs, uint32_t njobs, const vlb_bake_params* params,
                          const vlb_batch_schedule* sched);
/* Times the batch under candidate schedules (reps runs each, outputs written
 * every run), stores the fastest in the context for the batch's scene-size
 * class (later vlb_bake_batch calls with sched NULL and fused vlb_bake calls
 * on scenes of that class) and returns it with its mean milliseconds per
 * batch.  Tile walks: rays per lane per chunk 1, 2, 4, 8, 16 x job order.
 * Fused walks (VLB_PREC_FUSED): one knob at a time from the default -- CTAs
 * per SM (warps per SM) 7, 8, 9; node steps 2, 4, 6, 8, 12, 16; refill
 * threshold 8, 16, 24, 32; job order 0, 1 -- each kept at its fastest value
 * before the next is swept. */
vlb_status vlb_batch_autotune(vlb_ctx* ctx, const vlb_bake_job* jobs, uint32_t njobs, const vlb_bake_params* params,
                              uint32_t reps, vlb_batch_schedule* best, float* best_ms);
/* The trials of the context's last vlb_batch_autotune in the order run: up
 * to cap entries into out (may be NULL), their count in *n, the class the
 * winner was stored for in *size_class (0-3, may be NULL).  The first trial is
 * the default schedule. */
typedef struct vlb_tune_trial {
  vlb_batch_schedule schedule;
  float ms;
} vlb_tune_trial;
vlb_status vlb_batch_tune_log(const vlb_ctx* ctx, vlb_tune_trial* out, uint32_t cap, uint32_t* n,
                              uint32_t* size_class);

/* ---- bake service ------------------------------------------------------------
 * No reference counterpart (the reference bakes once per process,
 * src/baker/main.cpp:22-24).  A resident service over the scenes, direction sets
 * and skies of one context: requests are submitted from any thread, admitted
 * against a device-memory budget and baked by a worker thread in continuous
 * batches -- while one batch runs on the GPU the next is assembled from the
 * requests that arrived meanwhile and queued behind it (vlb_bake_batch
 * machinery on the service's own stream).  A bake may keep its primary hits
 * (triangle and distance per ray, 8 bytes); a relight of that bake re-shades
 * the kept hits with new sun and sky and re-traces only the shadow rays.
 * Every result is bit-identical to vlb_bake of the same request (a relight:
 * to vlb_bake of the original probes with the relight's parameters).
 * While a service runs, its context's objects may be used by other calls on
 * that context; they must outlive the requests that name them. */
typedef struct vlb_service vlb_service;
typedef struct vlb_service_config {
  uint64_t hbm_budget_bytes; /* device bytes for batches in flight plus kept hits (0: 64 GiB) */
  uint32_t lmax;             /* 2 or 3, every request */
  uint32_t precision;        /* vlb_precision of every request */
  uint32_t max_batch_probes; /* probes per batch (0: 1,048,576) */
  uint32_t max_inflight;     /* batches queued on the GPU at once (0: 2) */
  uint32_t slice_probes;     /* probes of one request per batch (0: 2048): a larger request is baked
                                in slices that share batches with the requests behind it */
} vlb_service_config;
typedef struct vlb_request {
  const vlb_scene* scene;         /* ignored by a relight (the original's) */
  const float* probe_xyz;         /* nprobes*3 host, copied at submit; ignored by a relight */
  uint32_t nprobes;               /* ignored by a relight */
  const vlb_bake_params* params;  /* lmax and precision come from the service; a relight keeps the
                                     original's direction set, tmin and tmax */
  uint64_t relight_of;            /* 0: bake; else the ticket of a bake submitted with keep_hits */
  uint32_t keep_hits;             /* 1: keep this bake's primary hits for relights */
} vlb_request;
/* The service's own state lives on ctx's device; ctx must outlive it. */
vlb_status vlb_service_create(vlb_ctx* ctx, const vlb_service_config* cfg, vlb_service** out);
/* Finishes the requests already submitted, then stops. */
void vlb_service_destroy(vlb_service* svc);
/* VLB_ERR_OOM: the request alone exceeds the budget.  *ticket > 0. */
vlb_status vlb_service_submit(vlb_service* svc, const vlb_request* req, uint64_t* ticket);
/* Waits up to timeout_ms (0: only look) for a ticket.  On VLB_OK, out (host,
 * nprobes x K x 3, may be NULL) gets the result, *latency_ms (may be NULL)
 * the time from submit to completion, and the ticket's result is released
 * (its kept hits stay until vlb_service_release or eviction).  VLB_ERR_TIMEOUT:
 * not done yet.  A failed request returns its error once. */
vlb_status vlb_service_wait(vlb_service* svc, uint64_t ticket, uint32_t timeout_ms, float* out, double* latency_ms);
/* Drops the kept hits of a bake (a later relight of it bakes in full). */
vlb_status vlb_service_release(vlb_service* svc, uint64_t ticket);
typedef struct vlb_service_stats {
  uint64_t submitted, completed, failed, batches;
  uint64_t relights, relights_rebaked; /* relights, and those whose kept hits were gone (baked in full) */
  uint64_t evictions;                  /* kept-hit sets dropped to admit work */
  uint64_t probes, rays;               /* completed work */
  uint64_t bytes_in_use, bytes_peak;   /* budget accounting: batches in flight + kept hits */
} vlb_service_stats;
vlb_status vlb_service_stats_read(vlb_service* svc, vlb_service_stats* out);
/* Message of the calling thread's last failed vlb_service_* call (never NULL). */
const char* vlb_service_last_error(void);
/* The admission rule of the service, as a pure host function (no GPU):
 * requests in queue order with their probe counts and device bytes are cut
 * into batches, each at most max_batch_probes probes (a larger request goes
 * alone) and at most budget_bytes (a request over the budget is refused,
 * batch size 0).  out_batch[i] = index of request i's batch (or UINT32_MAX
 * if refused); returns the number of batches in *nbatches.  The service
 * applies it to slices: a request over slice_probes enters as consecutive
 * slices, one per batch. */
vlb_status vlb_service_plan(const uint64_t* probes, const uint64_t* bytes, uint32_t n, uint64_t max_batch_probes,
                            uint64_t budget_bytes, uint32_t* out_batch, uint32_t* nbatches);

/* ---- projection and reconstruction ----------------------------------------
 * Replaces dispatchBakingKernel / shaders/sh.comp:23-42 for a radiance tile
 * laid out [nprobes][3][S] (S = the direction set's count): out nprobes x K x
 * 3.  dtype selects FP32 or BF16 radiance. */
typedef enum vlb_dtype {
  VLB_DTYPE_F32 = 0,
  VLB_DTYPE_BF16 = 1,       /* [nprobes][3][S] BF16 */
  VLB_DTYPE_BF16_SPLIT = 2  /* [nprobes][3][2S] BF16 hi/lo pairs: S high parts, then S low parts */
} vlb_dtype;
vlb_status vlb_project(vlb_ctx* ctx, const void* radiance, vlb_dtype dtype, uint32_t nprobes, const vlb_dirset* dirs,
                       uint32_t lmax, float* out);
/* Replaces shaders/sh_sum.comp:35-52: out[y][x] = scale * sum_k c_k
 * Y_k(toVector(x2phi(x), y2theta(y))) as w*h*3 FP32 (the reference uses
 * scale 1250). coeffs: K x 3. */
vlb_status vlb_sh_eval_envmap(vlb_ctx* ctx, const float* coeffs, uint32_t lmax, uint32_t w, uint32_t h, float scale,
                              float* out);

/* ---- baked-light glTF files ----------------------------------------------------
 * Host only (no GPU).  Replaces LightBaker::serialize
 * (src/baker/light_baker.cpp:375-401): the input glTF document plus one
 * buffer holding the coefficients as a base64 data URI, one bufferView over
 * it and the top-level "light" object {bufferView, gridStep {x, y, z},
 * lmax: coeff_count}, printed the way the reference's JSON library prints it
 * (every object's keys sorted, 4-space indentation) with a final newline --
 * the text the reference writes to baked_<name>.gltf.  coeffs: nprobes x
 * coeff_count x 3 FP32 (coeff_count 16 is the reference's layout and value).
 * out NULL: only *out_len (bytes including the terminating NUL). */
vlb_status vlb_gltf_write_light(const char* gltf_json, size_t json_len, const float* coeffs, uint32_t nprobes,
                                uint32_t coeff_count, const float grid_step[3], char* out, size_t out_cap,
                                size_t* out_len);
/* Replaces Scene_t::loadBakedLight (src/scene_manager.cpp:613-648): reads
 * gridStep, lmax (the coefficient count) and the coefficient bytes
 * (byteLength of the light's buffer) back.  A document without "light"
 * gives zeros and *coeffs_bytes = 0.  coeffs NULL: only the sizes. */
vlb_status vlb_gltf_read_light(const char* gltf_json, size_t json_len, float grid_step[3], uint32_t* coeff_count,
                               void* coeffs, size_t coeffs_cap, size_t* coeffs_bytes);
/* Scene geometry from a .gltf (external .bin or data-URI buffers) or .glb file,
 * host only.  Replaces the geometry side of Scene_t::loadNodes / loadNode /
 * fetchVertices / fetchIndices / loadMatrix (src/scene_manager.cpp:257-337,
 * 445-533, 860-870): the triangles of glTF scene 0 in world space (node
 * local matrix T*R*S*M, multiplied along the parent chain as the reference's
 * TLAS instances are), u8/u16/u32 indices, per-triangle albedo = the
 * material's baseColorFactor RGB (1 without a material; textures are not
 * sampled), bounds = the world AABB of the vertices (the reference's
 * getBounds also starts at the origin: vlb_scene_bounds(scene, 1, ...) gives
 * that form).  Only triangle primitives (mode 4). */
typedef struct vlb_gltf_mesh vlb_gltf_mesh;
vlb_status vlb_gltf_mesh_load(const char* path, vlb_gltf_mesh** out);
void vlb_gltf_mesh_free(vlb_gltf_mesh* mesh);
vlb_status vlb_gltf_mesh_info(const vlb_gltf_mesh* mesh, uint32_t* nverts, uint32_t* ntris, float bounds[6]);
/* positions nverts*3, indices ntris*3, albedo ntris*3 (any may be NULL) */
vlb_status vlb_gltf_mesh_get(const vlb_gltf_mesh* mesh, float* positions, uint32_t* indices, float* albedo);
/* vlb_gltf_mesh_load + vlb_scene_create in one call. */
vlb_status vlb_scene_create_gltf(vlb_ctx* ctx, const char* path, vlb_scene** out);
/* Message of the calling thread's last failed vlb_gltf_* call (never NULL). */
const char* vlb_gltf_last_error(void);

/* ---- evaluating a baked grid (the consumer side) --------------------------------
 * Replaces the probe lighting of shaders/main.rchit:124-168 with
 * shaders/sh.rmiss:23-39.  For each shading point x with normal n: the grid
 * cell holding x, its 8 corner probes, a visibility ray from x + bias*n toward
 * each probe (any hit in (0, |p - x|); scene NULL: all visible), weight
 * |step| - |p - x|, and out = sum(w E_p(n)) / sum(w) over the visible corners
 * with E_p(n) = sum_k c_pk Y_k(n).  The reference's faults are not reproduced:
 * its cell index assumes the grid starts at the origin and 7 x 7 x 7
 * probes in x-major order (the bake writes them breadth-first,
 * src/baker/light_baker.cpp:80-101), it strides by (16+1)^2 coefficients and sums 16
 * bands of a 16-coefficient probe, and it divides 0 by 0 when no probe is
 * visible (here: 0).  coeffs: the bake's output for the grid, nprobes x K x 3
 * in the reference's breadth-first order (vlb_probe_grid_ref_order).
 * vis_mask (may be NULL): bit c set when corner c (bit 2: +x, bit 1: +y,
 * bit 0: +z) was visible. */
typedef struct vlb_probe_grid {
  float origin[3];    /* position of probe (0,0,0): the bake bounds' minimum */
  float step[3];      /* grid step (light.gridStep) */
  uint32_t counts[3]; /* probes per axis */
} vlb_probe_grid;
vlb_status vlb_probe_eval(vlb_ctx* ctx, const vlb_scene* scene, const float* coeffs, uint32_t lmax,
                          const vlb_probe_grid* grid, const float* points, const float* normals, uint32_t n,
                          float shadow_bias, float* out_rgb, uint8_t* vis_mask);
/* Replaces shaders/skybox_sh.rmiss:14-25: out[i] = sum_k c_k Y_k(normalize(dirs[i]))
 * over K = (lmax+1)^2 coefficients (the reference sums 16 bands over a
 * 16-coefficient buffer). coeffs: K x 3. */
vlb_status vlb_sh_eval_dirs(vlb_ctx* ctx, const float* coeffs, uint32_t lmax, const float* dirs, uint32_t n,
                            float* out_rgb);

/* ---- debug env-map images ---------------------------------------------------------
 * The reference writes, for every probe, its traced equirect env map as an
 * R8G8B8A8 UNORM image (src/baker/env_map_generator.hpp:39) to "<probe>.png"
 * (src/baker/light_baker.cpp:306-307, EnvMapGenerator::saveImage
 * src/baker/env_map_generator.cpp:73-112); texels are sRGB-encoded by the shaders
 * (shaders/env_map.rchit:101, shaders/main.rmiss:40,
 * shaders/main.rchit:49-56) with alpha 1.
 * vlb_encode_rgba8: rgba[i] = UNORM8(srgb ? sRGB(scale*rgb[i]) : scale*rgb[i]),
 * alpha 255 (shaders/sh_sum.comp:51 is scale 1250 without sRGB).  Host or device. */
vlb_status vlb_encode_rgba8(vlb_ctx* ctx, const float* rgb, uint32_t n, float scale, uint32_t srgb, uint8_t* rgba);
/* One probe's env map as the reference's debug image: the probe's traced
 * radiance over params->dirs, which must be vlb_dirset_create_equirect(w, h)
 * (sample s = y*w + x is pixel (x, y)), sRGB-encoded into w x h RGBA8. */
vlb_status vlb_render_envmap(vlb_ctx* ctx, const vlb_scene* scene, const float probe_xyz[3],
                             const vlb_bake_params* params, uint32_t w, uint32_t h, uint8_t* rgba);
/* Host only: 8-bit RGBA PNG (stored deflate blocks) and binary PPM (alpha dropped). */
vlb_status vlb_image_write_png(const char* path, const uint8_t* rgba, uint32_t w, uint32_t h);
vlb_status vlb_image_write_ppm(const char* path, const uint8_t* rgba, uint32_t w, uint32_t h);
const char* vlb_image_last_error(void);

/* ---- synthetic inputs (bench and tests) -------------------------------------
 * Seeded SplitMix64 generators for the benchmark workloads.  The room is the
 * unit box [0,1]^3 open at +Y (10 triangles, albedo 0.5); each box has its
 * centre uniform in [0.1,0.9]^3, edges uniform in [0.05,0.2] per axis and
 * albedo uniform in [0.2,0.8] per channel (12 triangles).  Outputs: positions
 * (nverts*3), indices (ntris*3), per-triangle albedo (ntris*3); call with
 * NULL arrays to get the counts. */
vlb_status vlb_synth_box_scene(uint64_t seed, uint32_t nboxes, float* positions, uint32_t* indices, float* albedo,
                               uint32_t* nverts, uint32_t* ntris);
/* 6 x n x n RGB FP32 cubemap: 0.3 + three spherical Gaussian lobes, lobe
 * direction uniform on the sphere, sharpness uniform in [20,200], RGB
 * intensity uniform in [1,50]. */
vlb_status vlb_synth_cubemap(uint64_t seed, uint32_t n, float* out);
/* Unit direction uniform on the upper (+Y) hemisphere. */
vlb_status vlb_synth_sun(uint64_t seed, float out_dir[3]);

#ifdef __cplusplus
}
#endif
#endif /* VLB_H */
