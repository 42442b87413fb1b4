// vlb_api.cpp -- host C++ behind the C ABI of include/vlb.h.
//
// Replaces the reference's Vulkan host layer for the bake path
// (Application / SceneManager / SkyboxManager / LightBaker /
// EnvMapGenerator).  Everything here is orchestration: argument checks,
// staging of host arrays, scratch memory, kernel launches on the context's
// stream, error reporting.  All arithmetic on the bake path runs in the CUDA
// kernels of k_*.cu; there is no CPU fallback.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "vlb_internal.h"

namespace {

constexpr double kPiRef = 3.1415926538;  // shaders/sh_common.h:1
constexpr double kPi = 3.141592653589793;

vlb_status fail(vlb_ctx* ctx, vlb_status s, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return s;
}

vlb_status cuda_fail(vlb_ctx* ctx, cudaError_t e, const char* what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? VLB_ERR_OOM : VLB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define VLB_CUDA(ctx, call)                                   \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call); \
  } while (0)

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Grow-only named scratch buffer owned by the context.
vlb_status scratch(vlb_ctx* ctx, const char* name, size_t bytes, void** out) {
  auto& b = ctx->scratch[name];
  if (b.bytes < bytes) {
    if (b.p) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(b.p);
      b.p = nullptr;
      b.bytes = 0;
    }
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, VLB_ERR_OOM, "scratch '%s': cudaMalloc(%zu) failed", name, want);
    }
    b.bytes = want;
  }
  *out = b.p;
  return VLB_OK;
}

// A caller array on the device: used in place when it already is device
// memory, otherwise copied into named scratch.
vlb_status stage_in(vlb_ctx* ctx, const void* src, size_t bytes, const char* name, const void** dev) {
  if (bytes == 0) { *dev = nullptr; return VLB_OK; }
  if (is_device_ptr(src)) { *dev = src; return VLB_OK; }
  void* p;
  vlb_status st = scratch(ctx, name, bytes, &p);
  if (st) return st;
  VLB_CUDA(ctx, cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  ctx->host_inputs_pending = true;  // the call must not return before this copy has read src
  *dev = p;
  return VLB_OK;
}

struct OutBuf {
  void* user = nullptr;
  void* dev = nullptr;
  size_t bytes = 0;
  bool host = false;
};

vlb_status stage_out(vlb_ctx* ctx, void* user, size_t bytes, const char* name, OutBuf* o) {
  o->user = user; o->bytes = bytes;
  if (!user || bytes == 0) { o->dev = nullptr; return VLB_OK; }
  if (is_device_ptr(user)) { o->dev = user; o->host = false; return VLB_OK; }
  o->host = true;
  return scratch(ctx, name, bytes, &o->dev);
}

vlb_status copy_out(vlb_ctx* ctx, const OutBuf& o) {
  if (o.host && o.user && o.bytes)
    VLB_CUDA(ctx, cudaMemcpyAsync(o.user, o.dev, o.bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return VLB_OK;
}

// Clears and reports the device error counters h (a host copy of d_err taken
// on the synchronised stream).
vlb_status check_device_errors(vlb_ctx* ctx, const int* h) {
  bool any = false;
  for (int i = 0; i < vlbk::kErrSlots; ++i) any |= h[i] != 0;
  if (!any) return VLB_OK;
  VLB_CUDA(ctx, cudaMemset(ctx->d_err, 0, vlbk::kErrSlots * sizeof(int)));
  if (h[vlbk::kErrTimeout]) return fail(ctx, VLB_ERR_TIMEOUT, "a bounded device wait gave up (%d)", h[vlbk::kErrTimeout]);
  if (h[vlbk::kErrStackOverflow])
    return fail(ctx, VLB_ERR_INTERNAL, "BVH traversal stack overflow on %d rays", h[vlbk::kErrStackOverflow]);
  if (h[vlbk::kErrBounds])
    return fail(ctx, VLB_ERR_INTERNAL, "device bounds check failed on %d accesses", h[vlbk::kErrBounds]);
  return fail(ctx, VLB_ERR_INTERNAL, "device-side check failed (%d)", h[vlbk::kErrBadInput]);
}

vlb_status finish(vlb_ctx* ctx, bool sync) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "kernel launch");
  sync = sync || ctx->host_inputs_pending;
  ctx->host_inputs_pending = false;
  if (!sync) return VLB_OK;
  // the counters ride back behind the call's own copies: one synchronisation
  VLB_CUDA(ctx, cudaMemcpyAsync(ctx->h_err, ctx->d_err, vlbk::kErrSlots * sizeof(int), cudaMemcpyDeviceToHost,
                                ctx->stream));
  VLB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return check_device_errors(ctx, ctx->h_err);
}

// Brackets kernel launches with CUDA events when profiling is on.
struct KScope {
  vlb_ctx* ctx;
  std::string name;
  cudaEvent_t a = nullptr, b = nullptr;
  int nkernels;
  KScope(vlb_ctx* c, const char* n, int k = 1) : ctx(c), name(n), nkernels(k) {
    if (!ctx->profiling) return;
    a = take(); b = take();
    cudaEventRecord(a, ctx->stream);
  }
  cudaEvent_t take() {
    if (!ctx->event_pool.empty()) { cudaEvent_t e = ctx->event_pool.back(); ctx->event_pool.pop_back(); return e; }
    cudaEvent_t e; cudaEventCreate(&e); return e;
  }
  ~KScope() {
    ctx->launches += uint64_t(nkernels);
    if (!a) return;
    cudaEventRecord(b, ctx->stream);
    ctx->pending.push_back({name, a, b});
  }
};

void drain_profile(vlb_ctx* ctx) {
  for (auto& p : ctx->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      auto& s = ctx->stats[p.name];
      s.launches += 1;
      s.ms += ms;
    }
    ctx->event_pool.push_back(p.a);
    ctx->event_pool.push_back(p.b);
  }
  ctx->pending.clear();
  cudaGetLastError();
}

// ---- SH basis on the host (FP64), shaders/sh_common.h:26-116 ------------------
void sh_basis16(double x, double y, double z, double* o) {
  o[0] = 0.282095;
  o[1] = -0.488603 * y; o[2] = 0.488603 * z; o[3] = -0.488603 * x;
  o[4] = 1.092548 * x * y; o[5] = -1.092548 * y * z; o[6] = 0.315392 * (-x * x - y * y + 2.0 * z * z);
  o[7] = -1.092548 * x * z; o[8] = 0.546274 * (x * x - y * y);
  o[9] = -0.590044 * y * (3.0 * x * x - y * y); o[10] = 2.890611 * x * y * z;
  o[11] = -0.457046 * y * (4.0 * z * z - x * x - y * y);
  o[12] = 0.373176 * z * (2.0 * z * z - 3.0 * x * x - 3.0 * y * y);
  o[13] = -0.457046 * x * (4.0 * z * z - x * x - y * y);
  o[14] = 1.445306 * z * (x * x - y * y); o[15] = -0.590044 * x * (x * x - 3.0 * y * y);
}

// BF16 with round-to-nearest-even (finite inputs).
uint16_t bf16_rne(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return uint16_t(u >> 16);
}
float bf16_to_float(uint16_t h) {
  const uint32_t u = uint32_t(h) << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// Runs f(begin, end) over [0, n) split across up to 16 host threads (one
// range below `grain` items).  Every item's result depends on that item
// alone, so the output does not depend on the split; a thread that cannot be
// started runs its range on the calling thread.
template <class F>
void parallel_ranges(size_t n, size_t grain, F f) {
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const size_t parts = std::min<size_t>(hw, (n + grain - 1) / std::max<size_t>(grain, 1));
  if (parts <= 1) {
    f(size_t(0), n);
    return;
  }
  const size_t per = (n + parts - 1) / parts;
  std::vector<std::thread> th;
  for (size_t p = 1; p < parts; ++p) {
    const size_t b = p * per, e = std::min(n, b + per);
    if (b >= e) break;
    try {
      th.emplace_back(f, b, e);
    } catch (const std::system_error&) {
      f(b, e);
    }
  }
  f(size_t(0), std::min(n, per));
  for (auto& t : th) t.join();
}

// Builds the host + device halves of a direction set.
vlb_status dirset_finish(vlb_ctx* ctx, vlb_dirset* d, const std::vector<double>& bdirs, const std::vector<double>& w) {
  const uint32_t n = d->n;
  d->h_basis.assign(size_t(n) * 16, 0.0);
  d->h_basis32.assign(size_t(n) * 16, 0.f);
  std::vector<float> d4(size_t(n) * 4, 0.f), i4(size_t(n) * 4, 0.f);
  parallel_ranges(n, 1 << 16, [&](size_t b, size_t e) {
    for (size_t s = b; s < e; ++s) {
      double Y[16];
      sh_basis16(bdirs[3 * s], bdirs[3 * s + 1], bdirs[3 * s + 2], Y);
      for (int k = 0; k < 16; ++k) {
        d->h_basis[s * 16 + k] = w[s] * Y[k];
        d->h_basis32[s * 16 + k] = float(w[s] * Y[k]);
      }
      for (int a = 0; a < 3; ++a) {
        d4[4 * s + a] = d->h_dirs[3 * s + a];
        i4[4 * s + a] = vlbk::host_safe_inv(d->h_dirs[3 * s + a]);
      }
    }
  });
  VLB_CUDA(ctx, cudaMalloc(&d->d_dirs, size_t(n) * sizeof(float4)));
  VLB_CUDA(ctx, cudaMalloc(&d->d_dinv, size_t(n) * sizeof(float4)));
  VLB_CUDA(ctx, cudaMalloc(&d->d_basis16, size_t(n) * 16 * sizeof(float)));
  VLB_CUDA(ctx, cudaMemcpy(d->d_dirs, d4.data(), d4.size() * 4, cudaMemcpyHostToDevice));
  VLB_CUDA(ctx, cudaMemcpy(d->d_dinv, i4.data(), i4.size() * 4, cudaMemcpyHostToDevice));
  VLB_CUDA(ctx, cudaMemcpy(d->d_basis16, d->h_basis32.data(), d->h_basis32.size() * 4, cudaMemcpyHostToDevice));
  // trace order: directions grouped by ray octant (sign of 1/d per axis, as
  // the traversal sees it; warps in flight then share one traversal variant),
  // within an octant by a Morton code of the position on the octant's face
  // (|x|, |y| over |x| + |y| + |z|), so neighbouring positions are close
  // directions.  Outputs stay indexed by the caller's direction order.
  std::vector<uint32_t> order(n);
  auto oct = [&](uint32_t s) {
    int o = 0;
    for (int a = 0; a < 3; ++a) {
      const float c = d->h_dirs[3 * s + a];
      const bool neg = std::fabs(c) > 1e-30f ? c < 0.f : std::signbit(c);
      o |= neg ? (1 << a) : 0;
    }
    return o;
  };
  auto key = [&](uint32_t s) {
    const float ax = std::fabs(d->h_dirs[3 * s]), ay = std::fabs(d->h_dirs[3 * s + 1]),
                az = std::fabs(d->h_dirs[3 * s + 2]);
    const float l1 = ax + ay + az;
    const uint32_t u = l1 > 0.f ? uint32_t(std::min(1023.f, ax / l1 * 1023.f)) : 0u;
    const uint32_t v = l1 > 0.f ? uint32_t(std::min(1023.f, ay / l1 * 1023.f)) : 0u;
    uint32_t m = 0;
    for (int b = 0; b < 10; ++b) m |= (((u >> b) & 1u) << (2 * b)) | (((v >> b) & 1u) << (2 * b + 1));
    return (uint32_t(oct(s)) << 20) | m;  // 23 bits
  };
  std::vector<uint32_t> keys(n), tmp(n);
  parallel_ranges(n, 1 << 16, [&](size_t b, size_t e) {
    for (size_t s = b; s < e; ++s) keys[s] = key(uint32_t(s));
  });
  // stable LSD radix sort of the indices by key: 12 low bits, then 11 high
  for (uint32_t s = 0; s < n; ++s) order[s] = s;
  for (int pass = 0; pass < 2; ++pass) {
    const int shift = pass ? 12 : 0;
    std::vector<uint32_t> cnt(4097, 0);
    for (uint32_t s = 0; s < n; ++s) ++cnt[((keys[order[s]] >> shift) & 4095u) + 1];
    for (int b = 0; b < 4096; ++b) cnt[b + 1] += cnt[b];
    for (uint32_t s = 0; s < n; ++s) tmp[cnt[(keys[order[s]] >> shift) & 4095u]++] = order[s];
    order.swap(tmp);
  }
  VLB_CUDA(ctx, cudaMalloc(&d->d_order, size_t(n) * 4));
  VLB_CUDA(ctx, cudaMemcpy(d->d_order, order.data(), size_t(n) * 4, cudaMemcpyHostToDevice));
  // BF16 basis for the tensor-core projection, transposed [32][pitch]: row k
  // the BF16 rounding of w_s Y_k, row 16 + k the BF16 rounding of the rest
  d->bt_pitch = (n + 7) / 8 * 8;
  std::vector<uint16_t> bt(size_t(32) * d->bt_pitch, 0);
  parallel_ranges(n, 1 << 16, [&](size_t sb, size_t se) {
    for (size_t s = sb; s < se; ++s)
      for (int k = 0; k < 16; ++k) {
        const double b = d->h_basis[s * 16 + k];
        const uint16_t hi = bf16_rne(float(b));
        bt[size_t(k) * d->bt_pitch + s] = hi;
        bt[size_t(16 + k) * d->bt_pitch + s] = bf16_rne(float(b - double(bf16_to_float(hi))));
      }
  });
  VLB_CUDA(ctx, cudaMalloc(&d->d_bt, bt.size() * 2));
  VLB_CUDA(ctx, cudaMemcpy(d->d_bt, bt.data(), bt.size() * 2, cudaMemcpyHostToDevice));
  return VLB_OK;
}

// Panorama direction tables: per column (cos phi, sin phi), per row
// (sin theta, cos theta, pixel weight); sh_common.h:14-22, sh.comp:28-33,
// skybox_sh.comp:28 (phi - PI/2).
void pano_tables(uint32_t w, uint32_t h, bool shift, std::vector<float>& col, std::vector<float>& row) {
  col.assign(size_t(w) * 2, 0.f);
  row.assign(size_t(h) * 4, 0.f);
  const double area = (2.0 * kPiRef / w) * (kPiRef / h);
  for (uint32_t x = 0; x < w; ++x) {
    double phi = 2.0 * kPiRef * (double(x) + 0.5) / double(w);
    if (shift) phi -= kPiRef / 2.0;
    col[2 * x] = float(std::cos(phi));
    col[2 * x + 1] = float(std::sin(phi));
  }
  for (uint32_t y = 0; y < h; ++y) {
    const double th = kPiRef * (double(y) + 0.5) / double(h);
    row[4 * y] = float(std::sin(th));
    row[4 * y + 1] = float(std::cos(th));
    row[4 * y + 2] = float(area * std::sin(th));
  }
}

uint32_t k_of(uint32_t lmax) { return (lmax + 1) * (lmax + 1); }

struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // 24 random bits -> float in [0, 1), exact
  float uniform() { return float(next() >> 40) * 0x1p-24f; }
  float range(float lo, float hi) {
    volatile float span = hi - lo;
    volatile float t = span * uniform();
    return lo + t;
  }
  void unit_dir(double* d, bool upper) {
    for (;;) {
      const double x = 2.0 * uniform() - 1.0, y = 2.0 * uniform() - 1.0, z = 2.0 * uniform() - 1.0;
      const double r2 = x * x + y * y + z * z;
      if (r2 > 1.0 || r2 < 1e-6) continue;
      if (upper && y <= 0.0) continue;
      const double r = std::sqrt(r2);
      d[0] = x / r; d[1] = y / r; d[2] = z / r;
      return;
    }
  }
};

void cube_face_dir(int face, double u, double v, double* d) {
  switch (face) {
    case 0: d[0] = 1.0; d[1] = -v; d[2] = -u; break;
    case 1: d[0] = -1.0; d[1] = -v; d[2] = u; break;
    case 2: d[0] = u; d[1] = 1.0; d[2] = v; break;
    case 3: d[0] = u; d[1] = -1.0; d[2] = -v; break;
    case 4: d[0] = u; d[1] = -v; d[2] = 1.0; break;
    default: d[0] = -u; d[1] = -v; d[2] = -1.0; break;
  }
  const double n = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  d[0] /= n; d[1] /= n; d[2] /= n;
}

}  // namespace

extern "C" {

uint32_t vlb_version(void) { return VLB_VERSION; }

uint32_t vlb_build_flags(void) {
#ifdef VLB_BOUNDS_CHECK
  return VLB_BUILD_BOUNDS_CHECK;
#else
  return 0;
#endif
}

const char* vlb_status_string(vlb_status s) {
  switch (s) {
    case VLB_OK: return "ok";
    case VLB_ERR_INVALID: return "invalid argument";
    case VLB_ERR_OOM: return "out of memory";
    case VLB_ERR_TIMEOUT: return "timeout";
    case VLB_ERR_CUDA: return "cuda error";
    case VLB_ERR_UNSUPPORTED: return "unsupported";
    case VLB_ERR_INTERNAL: return "internal device check";
  }
  return "unknown";
}

// ---- context -------------------------------------------------------------------
vlb_status vlb_ctx_create(int device, vlb_ctx** out) {
  if (!out) return VLB_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return VLB_ERR_CUDA; }
  if (device < 0 || device >= ndev) return VLB_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return VLB_ERR_CUDA;
  vlb_ctx* c = new (std::nothrow) vlb_ctx();
  if (!c) return VLB_ERR_OOM;
  c->device = device;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->d_err, vlbk::kErrSlots * sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&c->h_err, vlbk::kErrSlots * sizeof(int)) != cudaSuccess ||
      cudaMemset(c->d_err, 0, vlbk::kErrSlots * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    vlb_ctx_destroy(c);
    return VLB_ERR_CUDA;
  }
  c->stream = c->own_stream;
  *out = c;
  return VLB_OK;
}

void vlb_ctx_destroy(vlb_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  drain_profile(ctx);
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  if (ctx->batch_exec) cudaGraphExecDestroy(ctx->batch_exec);
  for (auto& kv : ctx->scratch) cudaFree(kv.second.p);
  for (auto& kv : ctx->cube_sa) cudaFree(kv.second);
  for (auto& kv : ctx->cube_pt) cudaFree(kv.second);
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->h_err) cudaFreeHost(ctx->h_err);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

vlb_status vlb_ctx_set_stream(vlb_ctx* ctx, void* stream) {
  if (!ctx) return VLB_ERR_INVALID;
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return VLB_OK;
}

void* vlb_ctx_get_stream(vlb_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

vlb_status vlb_ctx_synchronize(vlb_ctx* ctx) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  return finish(ctx, true);
}

const char* vlb_last_error(const vlb_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

vlb_status vlb_ctx_set_profiling(vlb_ctx* ctx, int enable) {
  if (!ctx) return VLB_ERR_INVALID;
  ctx->profiling = enable != 0;
  return VLB_OK;
}

vlb_status vlb_ctx_profile_read(vlb_ctx* ctx, vlb_kernel_time* out, uint32_t cap, uint32_t* n) {
  if (!ctx || (!out && cap)) return VLB_ERR_INVALID;
  VLB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  drain_profile(ctx);
  uint32_t i = 0;
  for (auto& kv : ctx->stats) {
    if (i >= cap) break;
    std::memset(out[i].name, 0, sizeof out[i].name);
    std::strncpy(out[i].name, kv.first.c_str(), sizeof out[i].name - 1);
    out[i].launches = kv.second.launches;
    out[i].total_ms = kv.second.ms;
    ++i;
  }
  if (n) *n = i;
  return VLB_OK;
}

vlb_status vlb_ctx_profile_reset(vlb_ctx* ctx) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaStreamSynchronize(ctx->stream);
  drain_profile(ctx);
  ctx->stats.clear();
  return VLB_OK;
}

uint64_t vlb_ctx_launch_count(const vlb_ctx* ctx) { return ctx ? ctx->launches : 0; }

vlb_status vlb_ctx_test_hook(vlb_ctx* ctx, uint32_t hook, uint32_t wait_polls) {
  if (!ctx) return VLB_ERR_INVALID;
  if (hook > VLB_HOOK_HOLD_PRODUCER) return fail(ctx, VLB_ERR_INVALID, "test hook %u", hook);
  ctx->hold_producer = hook == VLB_HOOK_HOLD_PRODUCER ? 1u : 0u;
  ctx->wait_polls = hook ? wait_polls : 0u;
  return VLB_OK;
}

// ---- probe grid (light_baker.cpp:80-101) ---------------------------------------
vlb_status vlb_probe_grid_ref_order(const float bounds[6], const uint32_t counts[3], float* out_xyz,
                                    float grid_step[3]) {
  if (!bounds || !counts || !out_xyz) return VLB_ERR_INVALID;
  if (!counts[0] || !counts[1] || !counts[2]) return VLB_ERR_INVALID;
  float st[3];
  for (int a = 0; a < 3; ++a) {
    volatile float e = bounds[3 + a] - bounds[a];
    volatile float c = float(counts[a]) - 1.f;
    st[a] = e / c;
    if (grid_step) grid_step[a] = st[a];
  }
  size_t m = 1;
  out_xyz[0] = bounds[0]; out_xyz[1] = bounds[1]; out_xyz[2] = bounds[2];
  for (int dim = 0; dim < 3; ++dim) {
    const size_t prev = m;
    for (size_t q = 0; q < prev; ++q) {
      float p[3] = {out_xyz[3 * q], out_xyz[3 * q + 1], out_xyz[3 * q + 2]};
      for (uint32_t i = 0; i + 1 < counts[dim]; ++i) {
        volatile float v = p[dim] + st[dim];
        p[dim] = v;
        out_xyz[3 * m] = p[0]; out_xyz[3 * m + 1] = p[1]; out_xyz[3 * m + 2] = p[2];
        ++m;
      }
    }
  }
  return VLB_OK;
}

// ---- scene ----------------------------------------------------------------------------
vlb_status vlb_scene_create(vlb_ctx* ctx, const float* positions, uint32_t stride_bytes, uint32_t nverts,
                            const uint32_t* indices, uint32_t ntris, const float* tri_albedo, vlb_scene** out) {
  return vlb_scene_create_ex(ctx, positions, stride_bytes, nverts, indices, ntris, tri_albedo, 0, out);
}

vlb_status vlb_scene_create_ex(vlb_ctx* ctx, const float* positions, uint32_t stride_bytes, uint32_t nverts,
                               const uint32_t* indices, uint32_t ntris, const float* tri_albedo, uint32_t flags,
                               vlb_scene** out) {
  if (!ctx || !out) return VLB_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  if (stride_bytes < 12 || stride_bytes % 4) return fail(ctx, VLB_ERR_INVALID, "position stride %u", stride_bytes);
  if (ntris && (!positions || !indices || nverts == 0)) return fail(ctx, VLB_ERR_INVALID, "missing geometry");
  if (ntris > (1u << 30)) return fail(ctx, VLB_ERR_INVALID, "too many triangles (%u)", ntris);
  const uint32_t sf = stride_bytes / 4;
  // Host copies for validation and bounds (scene creation is not on the hot path).
  std::vector<float> hpos(size_t(nverts) * sf);
  std::vector<uint32_t> hidx(size_t(ntris) * 3);
  if (nverts) VLB_CUDA(ctx, cudaMemcpy(hpos.data(), positions, hpos.size() * 4, cudaMemcpyDefault));
  if (ntris) VLB_CUDA(ctx, cudaMemcpy(hidx.data(), indices, hidx.size() * 4, cudaMemcpyDefault));
  for (size_t i = 0; i < hidx.size(); ++i)
    if (hidx[i] >= nverts) return fail(ctx, VLB_ERR_INVALID, "index %u out of range at %zu", hidx[i], i);
  for (uint32_t v = 0; v < nverts; ++v)
    for (int a = 0; a < 3; ++a)
      if (!std::isfinite(hpos[size_t(v) * sf + a])) return fail(ctx, VLB_ERR_INVALID, "vertex %u is not finite", v);
  vlb_scene* sc = new (std::nothrow) vlb_scene();
  if (!sc) return VLB_ERR_OOM;
  sc->ctx = ctx; sc->ntris = ntris; sc->nverts = nverts;
  for (int a = 0; a < 3; ++a) { sc->bounds[a] = INFINITY; sc->bounds[3 + a] = -INFINITY; }
  for (uint32_t v = 0; v < nverts; ++v)
    for (int a = 0; a < 3; ++a) {
      sc->bounds[a] = std::min(sc->bounds[a], hpos[size_t(v) * sf + a]);
      sc->bounds[3 + a] = std::max(sc->bounds[3 + a], hpos[size_t(v) * sf + a]);
    }
  if (nverts == 0) for (int a = 0; a < 6; ++a) sc->bounds[a] = 0.f;
  if (ntris == 0) { *out = sc; return VLB_OK; }
  const uint32_t n = ntris;
  auto alloc = [&](void** p, size_t bytes) -> bool {
    if (cudaMalloc(p, std::max<size_t>(bytes, 16)) != cudaSuccess) { cudaGetLastError(); return false; }
    sc->bytes += bytes;
    return true;
  };
  float* dpos = nullptr; uint32_t* didx = nullptr; float* dalb = nullptr; void* scr = nullptr;
  bool ok = alloc((void**)&sc->codes, size_t(n) * 4) && alloc((void**)&sc->order, size_t(n) * 4) &&
            alloc((void**)&sc->child, size_t(2) * (n - 1 + (n == 1)) * 4) &&
            alloc((void**)&sc->box, size_t(2 * n - 1) * 6 * 4) &&
            alloc((void**)&sc->nodes, size_t(n - 1 + (n == 1)) * 64) && alloc((void**)&sc->tris, size_t(n) * 48) &&
            alloc((void**)&sc->albedo, size_t(n) * 16);
  const size_t scr_bytes = vlbk::lbvh_scratch_bytes(n);
  ok = ok && cudaMalloc((void**)&dpos, hpos.size() * 4) == cudaSuccess &&
       cudaMalloc((void**)&didx, hidx.size() * 4) == cudaSuccess &&
       (!tri_albedo || cudaMalloc((void**)&dalb, size_t(n) * 12) == cudaSuccess) &&
       cudaMalloc(&scr, scr_bytes) == cudaSuccess;
  vlb_status st = VLB_OK;
  if (!ok) {
    cudaGetLastError();
    st = fail(ctx, VLB_ERR_OOM, "scene allocation failed (%u triangles)", n);
  } else {
    cudaMemcpyAsync(dpos, hpos.data(), hpos.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(didx, hidx.data(), hidx.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (tri_albedo) cudaMemcpyAsync(dalb, tri_albedo, size_t(n) * 12, cudaMemcpyDefault, ctx->stream);
    vlbk::LbvhBuild b{};
    b.positions = dpos; b.stride_floats = sf; b.nverts = nverts; b.indices = didx; b.albedo = dalb; b.ntris = n;
    b.codes = sc->codes; b.order = sc->order; b.child = sc->child; b.box = sc->box; b.nodes = sc->nodes;
    b.tris = sc->tris; b.tri_albedo = sc->albedo; b.scratch = scr; b.scratch_bytes = scr_bytes;
    int launches = 0;
    {
      KScope k(ctx, "lbvh_build", 0);
      vlbk::launch_lbvh_build(b, ctx->stream, &launches);
      k.nkernels = launches;
    }
    if (n > 1 && !(flags & VLB_SCENE_TRAVERSAL_LBVH)) {
      void* pscr = nullptr;
      if (cudaMalloc(&pscr, vlbk::ploc_scratch_bytes(n)) != cudaSuccess) {
        cudaGetLastError();
        st = fail(ctx, VLB_ERR_OOM, "traversal tree scratch allocation failed (%u triangles)", n);
      } else {
        int pl = 0;
        KScope k(ctx, "ploc_build", 0);
        // a stalled clustering (1) keeps the LBVH already packed into sc->nodes
        if (vlbk::launch_ploc_build(sc->box + size_t(n - 1) * 6, n, sc->nodes, pscr, ctx->stream, &pl) < 0)
          st = fail(ctx, VLB_ERR_INTERNAL, "traversal tree build failed");
        k.nkernels = pl;
        cudaStreamSynchronize(ctx->stream);
        cudaFree(pscr);
      }
    }
    if (st == VLB_OK) st = finish(ctx, true);
    if (st == VLB_OK && (flags & VLB_SCENE_TRAVERSAL_WIDE)) st = vlbh::build_wide(ctx, sc);
    if (st == VLB_OK) st = vlbh::pair_siblings(ctx, sc);
  }
  cudaFree(dpos); cudaFree(didx); if (dalb) cudaFree(dalb); cudaFree(scr);
  if (st != VLB_OK) { vlb_scene_destroy(sc); return st; }
  *out = sc;
  return VLB_OK;
}

void vlb_scene_destroy(vlb_scene* s) {
  if (!s) return;
  if (s->ctx) { cudaSetDevice(s->ctx->device); cudaStreamSynchronize(s->ctx->stream); }
  cudaFree(s->codes); cudaFree(s->order); cudaFree(s->child); cudaFree(s->box);
  cudaFree(s->nodes); cudaFree(s->wnodes); cudaFree(s->tris); cudaFree(s->albedo);
  delete s;
}

uint32_t vlb_scene_triangle_count(const vlb_scene* s) { return s ? s->ntris : 0; }

vlb_status vlb_scene_bounds(const vlb_scene* s, int include_origin, float out[6]) {
  if (!s || !out) return VLB_ERR_INVALID;
  for (int a = 0; a < 6; ++a) out[a] = s->bounds[a];
  if (include_origin)
    for (int a = 0; a < 3; ++a) { out[a] = std::min(out[a], 0.f); out[3 + a] = std::max(out[3 + a], 0.f); }
  return VLB_OK;
}

vlb_status vlb_scene_bvh_export(const vlb_scene* s, uint32_t* codes, uint32_t* order, int32_t* children,
                                float* boxes) {
  if (!s) return VLB_ERR_INVALID;
  vlb_ctx* ctx = s->ctx;
  cudaSetDevice(ctx->device);
  VLB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const size_t n = s->ntris;
  if (n == 0) return VLB_OK;
  if (codes) VLB_CUDA(ctx, cudaMemcpy(codes, s->codes, n * 4, cudaMemcpyDefault));
  if (order) VLB_CUDA(ctx, cudaMemcpy(order, s->order, n * 4, cudaMemcpyDefault));
  if (children && n > 1) VLB_CUDA(ctx, cudaMemcpy(children, s->child, 2 * (n - 1) * 4, cudaMemcpyDefault));
  if (boxes) VLB_CUDA(ctx, cudaMemcpy(boxes, s->box, (2 * n - 1) * 24, cudaMemcpyDefault));
  return VLB_OK;
}

uint64_t vlb_scene_device_bytes(const vlb_scene* s) { return s ? s->bytes : 0; }

// ---- direction sets -------------------------------------------------------------------
vlb_status vlb_dirset_create_fibonacci(vlb_ctx* ctx, uint32_t n, vlb_frame frame, vlb_dirset** out) {
  if (!ctx || !out || n == 0 || (frame != VLB_FRAME_WORLD && frame != VLB_FRAME_XZY)) return VLB_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  vlb_dirset* d = new (std::nothrow) vlb_dirset();
  if (!d) return VLB_ERR_OOM;
  d->ctx = ctx; d->n = n;
  d->h_dirs.resize(size_t(n) * 3);
  std::vector<double> bd(size_t(n) * 3), w(n, 4.0 * kPi / double(n));
  const double g = 0.6180339887498949, two_pi = 6.283185307179586;
  parallel_ranges(n, 1 << 16, [&](size_t ib, size_t ie) {
    for (size_t i = ib; i < ie; ++i) {
      const double z = 1.0 - (2.0 * double(i) + 1.0) / double(n);
      const double r = std::sqrt(std::max(0.0, 1.0 - z * z));
      double fr = double(i) * g;
      fr -= std::floor(fr);
      const double phi = two_pi * fr;
      const float f[3] = {float(r * std::cos(phi)), float(r * std::sin(phi)), float(z)};
      for (int a = 0; a < 3; ++a) d->h_dirs[3 * i + a] = f[a];
      if (frame == VLB_FRAME_WORLD) { bd[3 * i] = f[0]; bd[3 * i + 1] = f[1]; bd[3 * i + 2] = f[2]; }
      else { bd[3 * i] = f[0]; bd[3 * i + 1] = f[2]; bd[3 * i + 2] = f[1]; }
    }
  });
  vlb_status st = dirset_finish(ctx, d, bd, w);
  if (st) { vlb_dirset_destroy(d); return st; }
  *out = d;
  return VLB_OK;
}

vlb_status vlb_dirset_create_equirect(vlb_ctx* ctx, uint32_t w, uint32_t h, vlb_dirset** out) {
  if (!ctx || !out || !w || !h || uint64_t(w) * h > (1u << 28)) return VLB_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  vlb_dirset* d = new (std::nothrow) vlb_dirset();
  if (!d) return VLB_ERR_OOM;
  const uint32_t n = w * h;
  d->ctx = ctx; d->n = n;
  d->h_dirs.resize(size_t(n) * 3);
  std::vector<double> bd(size_t(n) * 3), wt(n);
  parallel_ranges(h, std::max<size_t>(1, (1 << 16) / w), [&](size_t yb, size_t ye) {
    for (size_t y = yb; y < ye; ++y)
      for (uint32_t x = 0; x < w; ++x) {
        const size_t s = y * w + x;
        const double phi = 2.0 * kPiRef * (double(x) + 0.5) / double(w);
        const double th = kPiRef * (double(y) + 0.5) / double(h);
        const double r = std::sin(th);
        double v[3] = {r * std::cos(phi), r * std::sin(phi), std::cos(th)};
        const double nn = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int a = 0; a < 3; ++a) v[a] /= nn;
        d->h_dirs[3 * s] = float(v[0]); d->h_dirs[3 * s + 1] = float(v[2]); d->h_dirs[3 * s + 2] = float(v[1]);
        bd[3 * s] = v[0]; bd[3 * s + 1] = v[1]; bd[3 * s + 2] = v[2];
        wt[s] = (2.0 * kPiRef / w) * (kPiRef / h) * std::sin(th);
      }
  });
  vlb_status st = dirset_finish(ctx, d, bd, wt);
  if (st) { vlb_dirset_destroy(d); return st; }
  *out = d;
  return VLB_OK;
}

vlb_status vlb_dirset_create(vlb_ctx* ctx, const float* trace_dirs, const float* basis_dirs, const double* weights,
                             uint32_t n, vlb_dirset** out) {
  if (!ctx || !out || !trace_dirs || !weights || n == 0) return VLB_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  vlb_dirset* d = new (std::nothrow) vlb_dirset();
  if (!d) return VLB_ERR_OOM;
  d->ctx = ctx; d->n = n;
  d->h_dirs.assign(trace_dirs, trace_dirs + size_t(n) * 3);
  std::vector<double> bd(size_t(n) * 3), w(weights, weights + n);
  const float* b = basis_dirs ? basis_dirs : trace_dirs;
  for (size_t i = 0; i < size_t(n) * 3; ++i) bd[i] = b[i];
  vlb_status st = dirset_finish(ctx, d, bd, w);
  if (st) { vlb_dirset_destroy(d); return st; }
  *out = d;
  return VLB_OK;
}

void vlb_dirset_destroy(vlb_dirset* d) {
  if (!d) return;
  if (d->ctx) { cudaSetDevice(d->ctx->device); cudaStreamSynchronize(d->ctx->stream); }
  cudaFree(d->d_dirs);
  cudaFree(d->d_dinv);
  cudaFree(d->d_basis16);
  cudaFree(d->d_order);
  cudaFree(d->d_bt);
  cudaFree(d->d_bt2);
  delete d;
}

uint32_t vlb_dirset_count(const vlb_dirset* d) { return d ? d->n : 0; }

vlb_status vlb_dirset_export(const vlb_dirset* d, float* trace_dirs, float* basis) {
  if (!d) return VLB_ERR_INVALID;
  vlb_ctx* ctx = d->ctx;
  cudaSetDevice(ctx->device);
  if (trace_dirs) {
    std::vector<float> d4(size_t(d->n) * 4);
    VLB_CUDA(ctx, cudaMemcpy(d4.data(), d->d_dirs, d4.size() * 4, cudaMemcpyDeviceToHost));
    for (uint32_t s = 0; s < d->n; ++s)
      for (int a = 0; a < 3; ++a) trace_dirs[3 * s + a] = d4[4 * s + a];
  }
  if (basis) VLB_CUDA(ctx, cudaMemcpy(basis, d->d_basis16, size_t(d->n) * 64, cudaMemcpyDeviceToHost));
  return VLB_OK;
}

// ---- skybox SH ---------------------------------------------------------------------------
static vlb_status cube_pair_table(vlb_ctx* ctx, uint32_t n, uint32_t lmax, const float2** out) {
  const uint64_t key = (uint64_t(n) << 8) | lmax;
  auto it = ctx->cube_pt.find(key);
  if (it != ctx->cube_pt.end()) { *out = it->second; return VLB_OK; }
  float2* p = nullptr;
  VLB_CUDA(ctx, cudaMalloc(&p, vlbk::cube_pair_table_bytes(n, lmax)));
  {
    KScope k(ctx, "cube_pair_table");
    vlbk::launch_cube_pair_table(p, n, lmax, ctx->stream);
  }
  ctx->cube_pt[key] = p;
  *out = p;
  return VLB_OK;
}

static vlb_status cube_sa_table(vlb_ctx* ctx, uint32_t n, const float** out) {
  auto it = ctx->cube_sa.find(n);
  if (it != ctx->cube_sa.end()) { *out = it->second; return VLB_OK; }
  float* p = nullptr;
  VLB_CUDA(ctx, cudaMalloc(&p, size_t(n) * n * 4));
  {
    KScope k(ctx, "cube_solid_angle");
    vlbk::launch_cube_solid_angle(p, n, ctx->stream);
  }
  ctx->cube_sa[n] = p;
  *out = p;
  return VLB_OK;
}

vlb_status vlb_skybox_sh_batched(vlb_ctx* ctx, const void* texels, vlb_texel_format fmt, vlb_sky_layout layout,
                                 uint32_t w, uint32_t h, uint32_t count, uint32_t lmax, uint32_t flags, float* out) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (!texels || !out) return fail(ctx, VLB_ERR_INVALID, "null texels or output");
  if (lmax != 2 && lmax != 3) return fail(ctx, VLB_ERR_INVALID, "lmax must be 2 or 3 (got %u)", lmax);
  if (fmt != VLB_TEXEL_RGB32F && fmt != VLB_TEXEL_RGBA8) return fail(ctx, VLB_ERR_INVALID, "texel format %d", fmt);
  if (layout != VLB_SKY_CUBEMAP && layout != VLB_SKY_PANORAMA && layout != VLB_SKY_ENVMAP)
    return fail(ctx, VLB_ERR_INVALID, "layout %d", layout);
  if (!w || !h || !count) return fail(ctx, VLB_ERR_INVALID, "empty image");
  if (layout == VLB_SKY_CUBEMAP && w != h) return fail(ctx, VLB_ERR_INVALID, "cubemap faces must be square");
  const uint64_t T64 = layout == VLB_SKY_CUBEMAP ? 6ull * w * w : uint64_t(w) * h;
  if (T64 >= (1ull << 31) || T64 * count >= (1ull << 40)) return fail(ctx, VLB_ERR_INVALID, "image too large");
  const uint32_t T = uint32_t(T64);
  const uint32_t TB = fmt == VLB_TEXEL_RGB32F ? 12 : 4;
  const uint32_t K = k_of(lmax), V = 3 * K;
  const void* dtex;
  vlb_status st = stage_in(ctx, texels, size_t(T) * count * TB, "sky_in", &dtex);
  if (st) return st;
  vlbk::SkyboxArgs a{};
  a.texels = dtex; a.fmt = fmt; a.layout = layout; a.w = w; a.h = h; a.count = count; a.lmax = lmax;
  a.flags = flags; a.texels_per_map = T; a.err = ctx->d_err;
  a.hold_producer = ctx->hold_producer; a.wait_polls = ctx->wait_polls;
  if (layout == VLB_SKY_CUBEMAP) {
    st = cube_sa_table(ctx, w, &a.solid_angle);
    // faces up to 1024: the texel-pair basis table (6n^2 x 36-64 B), the
    // group kernel (8 maps per basis row)
    if (!st && w <= 1024) st = cube_pair_table(ctx, w, lmax, &a.pair_table);
    if (st) return st;
  } else {
    std::vector<float> col, row;
    pano_tables(w, h, layout == VLB_SKY_PANORAMA, col, row);
    void *dc, *dr;
    if ((st = scratch(ctx, "pano_col", col.size() * 4, &dc)) || (st = scratch(ctx, "pano_row", row.size() * 4, &dr)))
      return st;
    VLB_CUDA(ctx, cudaMemcpyAsync(dc, col.data(), col.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    VLB_CUDA(ctx, cudaMemcpyAsync(dr, row.data(), row.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    VLB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // host vectors go out of scope
    a.col_tab = static_cast<const float2*>(dc);
    a.row_tab = static_cast<const float4*>(dr);
  }
  vlbk::skybox_plan(a, 0);
  const uint32_t spm = a.slabs_per_map;
  void* part;
  if ((st = scratch(ctx, "sky_partial", size_t(count) * spm * vlbk::kSkyPartialsPerSlab * V * 4, &part))) return st;
  a.partial = static_cast<float*>(part);
  const bool tma = (reinterpret_cast<uintptr_t>(dtex) % 16 == 0) && ((uint64_t(T) * TB) % 16 == 0);
  OutBuf ob;
  if ((st = stage_out(ctx, out, size_t(count) * V * 4, "sky_out", &ob))) return st;
  int per_map;
  {
    KScope k(ctx, tma ? (a.pair_table ? "skybox_cube_group" : "skybox_sh_tma") : "skybox_sh");
    per_map = vlbk::launch_skybox_sh(a, tma, ctx->num_sms, ctx->stream);
  }
  {
    KScope k(ctx, "sh_finalize");
    vlbk::launch_sh_finalize(a.partial, count, uint32_t(per_map), V, static_cast<float*>(ob.dev), ctx->stream);
  }
  if ((st = copy_out(ctx, ob))) return st;
  return finish(ctx, ob.host);
}

vlb_status vlb_skybox_sh(vlb_ctx* ctx, const void* texels, vlb_texel_format fmt, vlb_sky_layout layout, uint32_t w,
                         uint32_t h, uint32_t lmax, uint32_t flags, float* out) {
  return vlb_skybox_sh_batched(ctx, texels, fmt, layout, w, h, 1, lmax, flags, out);
}

vlb_status vlb_sky_create(vlb_ctx* ctx, const float* cubemap_rgb, uint32_t n, vlb_sky** out) {
  if (!ctx || !out || !cubemap_rgb || n == 0 || n > 16384) return VLB_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  vlb_sky* s = new (std::nothrow) vlb_sky();
  if (!s) return VLB_ERR_OOM;
  s->ctx = ctx; s->n = n;
  const size_t bytes = size_t(6) * n * n * 12;
  if (cudaMalloc(&s->d_texels, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete s;
    return fail(ctx, VLB_ERR_OOM, "sky allocation");
  }
  if (cudaMemcpy(s->d_texels, cubemap_rgb, bytes, cudaMemcpyDefault) != cudaSuccess) {
    cudaGetLastError();
    vlb_sky_destroy(s);
    return fail(ctx, VLB_ERR_CUDA, "sky upload");
  }
  *out = s;
  return VLB_OK;
}

void vlb_sky_destroy(vlb_sky* s) {
  if (!s) return;
  if (s->ctx) { cudaSetDevice(s->ctx->device); cudaStreamSynchronize(s->ctx->stream); }
  cudaFree(s->d_texels);
  delete s;
}

// ---- bake ------------------------------------------------------------------------------------
void vlb_bake_params_default(vlb_bake_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->lmax = 3;
  p->precision = VLB_PREC_FP32;
  p->sun_dir[0] = 0.f; p->sun_dir[1] = 1.f; p->sun_dir[2] = 0.f;
  p->sun_intensity = 5.f;
  p->tmin = 0.001f; p->tmax = 10000.f;
  p->shadow_bias = 0.005f;
  p->shading = VLB_SHADE_LAMBERT_SUN;
  p->light_pos[0] = 1.f; p->light_pos[1] = 10.f; p->light_pos[2] = 1.f;  // shaders/env_map.rchit:25
}

// The BF16 basis of a direction set for hi/lo split tiles ([32][2S]): built
// on the host from the FP64 basis on first use (synchronous; never inside a
// stream capture: callers make it before they enqueue).
static vlb_status dirset_split_basis(vlb_ctx* ctx, const vlb_dirset* d) {
  std::lock_guard<std::mutex> g(d->bt2_mu);
  if (d->d_bt2) return VLB_OK;
  const uint32_t n = d->n;
  const uint32_t pitch = (2 * n + 7) / 8 * 8;
  std::vector<uint16_t> bt(size_t(32) * pitch, 0);
  parallel_ranges(n, 1 << 16, [&](size_t sb, size_t se) {
    for (size_t s = sb; s < se; ++s)
      for (int k = 0; k < 16; ++k) {
        const double b = d->h_basis[s * 16 + k];
        const uint16_t hi = bf16_rne(float(b));
        const uint16_t lo = bf16_rne(float(b - double(bf16_to_float(hi))));
        bt[size_t(k) * pitch + s] = hi;       // x radiance hi
        bt[size_t(k) * pitch + n + s] = hi;   // x radiance lo
        bt[size_t(16 + k) * pitch + s] = lo;  // x radiance hi (lo x lo is dropped)
      }
  });
  uint16_t* dev = nullptr;
  VLB_CUDA(ctx, cudaMalloc(&dev, bt.size() * 2));
  const cudaError_t e = cudaMemcpy(dev, bt.data(), bt.size() * 2, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { cudaFree(dev); return cuda_fail(ctx, e, "split basis upload"); }
  d->bt2_pitch = pitch;
  d->d_bt2 = dev;
  return VLB_OK;
}

// BF16 tile projection: the tcgen05 kernel when the tile meets its alignment
// (columns a multiple of 8, 16-byte aligned), else the CUDA-core kernel.
// split: the tile holds hi/lo pairs ([rows][2S]); the tensor-core form then
// runs K = 2S against the split basis, so out = hi*bhi + lo*bhi + hi*blo.
// `part_name`: the scratch for split partials (the batch path, whose launches
// a CUDA graph may replay, keeps its own).  Split tiles need
// dirset_split_basis first.
static vlb_status project_bf16(vlb_ctx* ctx, const uint16_t* rad, uint32_t nprobes, const vlb_dirset* dirs,
                               uint32_t K, float* out, bool split, const char* part_name = "project_partial") {
  const uint32_t S = dirs->n;
  if (vlbk::project_tc_supported(rad, split ? 2 * S : S) && (!split || dirs->d_bt2)) {
    KScope k(ctx, split ? "project_tc_split" : "project_tc");
    const int r = split ? vlbk::launch_project_tc(rad, nprobes, 2 * S, dirs->d_bt2, dirs->bt2_pitch, K, out,
                                                  ctx->d_err, ctx->num_sms, ctx->stream, ctx->hold_producer,
                                                  ctx->wait_polls)
                        : vlbk::launch_project_tc(rad, nprobes, S, dirs->d_bt, dirs->bt_pitch, K, out, ctx->d_err,
                                                  ctx->num_sms, ctx->stream, ctx->hold_producer, ctx->wait_polls);
    if (r < 0) return fail(ctx, VLB_ERR_CUDA, "tensor map encoding failed for the BF16 projection");
    return VLB_OK;
  }
  void* part = nullptr;
  const size_t pb = vlbk::project_partial_bytes(nprobes, S, K);
  if (pb) {
    vlb_status st = scratch(ctx, part_name, pb, &part);
    if (st) return st;
  }
  KScope k(ctx, "project_bf16", pb ? 2 : 1);
  vlbk::launch_project_bf16_simt(rad, nprobes, S, dirs->d_basis16, K, out, static_cast<float*>(part), split ? 1 : 0,
                                 ctx->stream);
  return VLB_OK;
}

// FP32 tile projection (k_project; few-row tiles split along the samples).
static vlb_status project_f32(vlb_ctx* ctx, const float* rad, uint32_t nprobes, const vlb_dirset* dirs, uint32_t K,
                              float* out, const char* part_name = "project_partial") {
  void* part = nullptr;
  const size_t pb = vlbk::project_partial_bytes(nprobes, dirs->n, K);
  if (pb) {
    vlb_status st = scratch(ctx, part_name, pb, &part);
    if (st) return st;
  }
  KScope k(ctx, "project_f32", pb ? 2 : 1);
  vlbk::launch_project_f32(rad, nprobes, dirs->n, dirs->d_basis16, K, out, static_cast<float*>(part), ctx->stream,
                           ctx->d_err, ctx->num_sms, ctx->hold_producer, ctx->wait_polls);
  return VLB_OK;
}

// Common part of a bake launch: validated parameters -> trace arguments,
// probes staged on the device and sorted into spatially compact packets.
// Traversal mode of one bake: packets only when the flag asks for them.  The
// lane walk (per-lane state machines, rays of one probe fetched together)
// is faster on every box scene measured, 200 to 200k triangles with 64 to
// 32k probes (1.04x on 32k probes in 200 triangles to 8.6x on 64 probes in
// 200k triangles; 262,144 grid probes x 1024 directions in 49k triangles:
// 179 ms against 242 ms).
static uint32_t lane_mode(const vlb_scene*, uint32_t, uint32_t flags, uint32_t shading) {
  if (shading == VLB_SHADE_REF_PHONG) return 1;  // the reference's shading is built into the lane walks
  return (flags & VLB_BAKE_TRAVERSAL_PACKET) && !(flags & VLB_BAKE_TRAVERSAL_LANE) ? 0 : 1;
}

// Grid mode (per-direction triangle grids) runs when the grid flag asks for
// it and the scene qualifies (at most kGridMaxTris triangles, grids within
// 2 GB).  It is not chosen by default: building S+1 grids per bake costs
// more than it saves on the configurations measured (one grid-build CTA
// takes ~0.15 ms for 778 triangles; 4096 grid probes x 256 directions trace
// in 0.19 ms against the lane walk's 0.21 ms).
static uint32_t grid_cells_per_side(uint32_t ntris) { return ntris <= 1024 ? 32 : 16; }

static bool grid_mode(const vlb_scene* scene, uint32_t nprobes, uint32_t S, const vlb_bake_params* p) {
  const uint32_t T = scene->ntris;
  if (!vlbk::grid_supported(T, nprobes, S)) return false;
  const uint64_t G = grid_cells_per_side(T);
  const uint64_t bytes = uint64_t(S + 1) * (64 + (G * G + 1) * 4 + uint64_t(vlbk::kGridCap) * 2 + uint64_t(T) * 24);
  if (bytes > (2ull << 30)) return false;
  return (p->flags & VLB_BAKE_TRAVERSAL_GRID) && !(p->flags & VLB_BAKE_FORCE_FUSED_KERNEL) &&
         p->shading == VLB_SHADE_LAMBERT_SUN;  // the grids hold the sun's parallel shadow rays
}

// Checks the parameters of one bake; *sun_len gets |sun_dir| (FP64).
static vlb_status check_params(vlb_ctx* ctx, const vlb_scene* scene, const vlb_bake_params* p, double* sun_len) {
  if (!scene || !p || !p->dirs) return fail(ctx, VLB_ERR_INVALID, "scene, params and params->dirs are required");
  auto mine = [ctx](const vlb_ctx* c) { return c == ctx || (ctx->parent && c == ctx->parent); };
  if (!mine(scene->ctx) || !mine(p->dirs->ctx) || (p->sky && !mine(p->sky->ctx)))
    return fail(ctx, VLB_ERR_INVALID, "handles belong to another context");
  if (p->lmax != 2 && p->lmax != 3) return fail(ctx, VLB_ERR_INVALID, "lmax must be 2 or 3 (got %u)", p->lmax);
  if (p->precision > VLB_PREC_BF16) return fail(ctx, VLB_ERR_INVALID, "precision %u", p->precision);
  const double sl = std::sqrt(double(p->sun_dir[0]) * p->sun_dir[0] + double(p->sun_dir[1]) * p->sun_dir[1] +
                              double(p->sun_dir[2]) * p->sun_dir[2]);
  if (!(sl > 0.0) || !std::isfinite(sl)) return fail(ctx, VLB_ERR_INVALID, "sun direction must be non-zero");
  if (!(p->tmax > p->tmin) || p->tmin < 0.f) return fail(ctx, VLB_ERR_INVALID, "bad ray interval");
  if (p->shading > VLB_SHADE_REF_PHONG) return fail(ctx, VLB_ERR_INVALID, "shading %u", p->shading);
  if (p->shading == VLB_SHADE_REF_PHONG &&
      !(std::isfinite(p->light_pos[0]) && std::isfinite(p->light_pos[1]) && std::isfinite(p->light_pos[2])))
    return fail(ctx, VLB_ERR_INVALID, "light position must be finite");
  if (p->shading == VLB_SHADE_REF_PHONG && (p->flags & VLB_BAKE_FORCE_FUSED_KERNEL))
    return fail(ctx, VLB_ERR_UNSUPPORTED, "the packet fused kernel has the sun's shading only");
  *sun_len = sl;
  return VLB_OK;
}

static vlb_status prepare_trace(vlb_ctx* ctx, const vlb_scene* scene, const float* probe_xyz, uint32_t nprobes,
                                const vlb_bake_params* p, vlbk::TraceArgs* out) {
  double sl = 0.0;
  vlb_status st = check_params(ctx, scene, p, &sl);
  if (st) return st;
  if (!probe_xyz) return fail(ctx, VLB_ERR_INVALID, "null probes");
  const void* dprobes;
  if ((st = stage_in(ctx, probe_xyz, size_t(nprobes) * 12, "probes_in", &dprobes))) return st;
  void *order, *oscr, *wc;
  if ((st = scratch(ctx, "probe_order", size_t(nprobes) * 4, &order)) ||
      (st = scratch(ctx, "probe_order_tmp", vlbk::probe_order_scratch_bytes(nprobes), &oscr)) ||
      (st = scratch(ctx, "trace_work", 256, &wc)))
    return st;
  {
    float b[6];
    for (int a = 0; a < 6; ++a) b[a] = scene->bounds[a];
    KScope k(ctx, "probe_order", 0);
    k.nkernels = vlbk::launch_probe_order(static_cast<const float*>(dprobes), nprobes, b,
                                          static_cast<uint32_t*>(order), oscr, static_cast<uint32_t*>(wc),
                                          ctx->stream);
  }
  vlbk::TraceArgs& a = *out;
  a = vlbk::TraceArgs{};
  a.nodes = scene->nodes; a.tris = scene->tris; a.albedo = scene->albedo; a.ntris = scene->ntris;
  a.wnodes = scene->wnodes;
  a.nwide = scene->nwide;
  a.probes = static_cast<const float*>(dprobes); a.nprobes = nprobes;
  a.order = static_cast<const uint32_t*>(order);
  a.dirs = p->dirs->d_dirs; a.dir_order = p->dirs->d_order; a.S = p->dirs->n;
  a.sun = make_float3(float(p->sun_dir[0] / sl), float(p->sun_dir[1] / sl), float(p->sun_dir[2] / sl));
  a.sun_inv = make_float3(vlbk::host_safe_inv(a.sun.x), vlbk::host_safe_inv(a.sun.y), vlbk::host_safe_inv(a.sun.z));
  a.dinv = p->dirs->d_dinv;
  a.sun_scale = float(double(p->sun_intensity) / kPi);
  a.tmin = p->tmin; a.tmax = p->tmax; a.bias = p->shadow_bias;
  a.sky = p->sky ? p->sky->d_texels : nullptr; a.sky_n = p->sky ? p->sky->n : 0;
  a.basis16 = p->dirs->d_basis16; a.K = k_of(p->lmax); a.err = ctx->d_err;
  a.lane = lane_mode(scene, nprobes, p->flags, p->shading);
  a.shading = p->shading;
  a.light = make_float3(p->light_pos[0], p->light_pos[1], p->light_pos[2]);
  if (grid_mode(scene, nprobes, a.S, p)) {
    const uint32_t G = grid_cells_per_side(scene->ntris), T = scene->ntris;
    const size_t n = size_t(a.S) + 1;
    void *hdr, *cells, *ent, *box, *dep;
    if ((st = scratch(ctx, "grid_hdr", n * 64, &hdr)) ||
        (st = scratch(ctx, "grid_cells", n * (size_t(G) * G + 1) * 4, &cells)) ||
        (st = scratch(ctx, "grid_ent", n * vlbk::kGridCap * 2, &ent)) ||
        (st = scratch(ctx, "grid_box", n * T * 16, &box)) || (st = scratch(ctx, "grid_dep", n * T * 8, &dep)))
      return st;
    a.grid_hdr = static_cast<float4*>(hdr);
    a.grid_cells = static_cast<uint32_t*>(cells);
    a.grid_ent = static_cast<uint16_t*>(ent);
    a.grid_box = static_cast<float4*>(box);
    a.grid_dep = static_cast<float2*>(dep);
    a.grid_g = G;
    float L = 1e-30f;
    for (int k = 0; k < 6; ++k) L = std::max(L, std::fabs(scene->bounds[k]));
    a.grid_margin = L * 0x1p-12f;
    a.grid_far = 256.f * L;
    KScope k(ctx, "grid_build");
    vlbk::launch_grid_build(a, ctx->stream);
  }
  vlbk::plan_trace(a, ctx->num_sms, p->precision == VLB_PREC_FUSED);
  a.work_counter = static_cast<uint32_t*>(wc);  // zeroed by the probe-order launch
  return VLB_OK;
}

// Scene-size class of a triangle count: under 4K, 64K, 1M triangles, or more.
static uint32_t size_class(uint32_t ntris) {
  return ntris < 4096 ? 0u : ntris < 65536 ? 1u : ntris < (1u << 20) ? 2u : 3u;
}
static uint32_t batch_class(const vlb_bake_job* jobs, uint32_t njobs) {
  uint32_t m = 0;
  for (uint32_t i = 0; i < njobs; ++i)
    if (jobs[i].scene) m = std::max(m, jobs[i].scene->ntris);
  return size_class(m);
}
// The tuned schedule of a class, else the library default.
static vlb_batch_schedule class_sched(const vlb_ctx* ctx, uint32_t cls) {
  return ctx->tuned_set[cls] ? ctx->tuned[cls] : vlb_batch_schedule{0, 1, 1, 0, 0, 0};
}

// The fused walk's launch knobs of a schedule (0: the library default).
static vlbk::FusedSched fused_sched(const vlb_batch_schedule& sc) {
  vlbk::FusedSched f;
  if (sc.ctas_per_sm) f.ctas_per_sm = sc.ctas_per_sm;
  if (sc.node_steps) f.node_steps = sc.node_steps;
  if (sc.refill_idle) f.refill_idle = sc.refill_idle;
  return f;
}

// The scene, shading, probe and direction fields of one bake as a job of the
// fused lane walk (the fused-projection fields are set by the caller).
static void job_from_trace(const vlbk::TraceArgs& a, vlbk::BakeJobDev* j) {
  j->nodes = a.nodes; j->wnodes = a.wnodes; j->tris = a.tris; j->albedo = a.albedo; j->ntris = a.ntris;
  j->nwide = a.nwide;
  j->tmin = a.tmin; j->tmax = a.tmax; j->bias = a.bias;
  j->sun = a.sun; j->sun_inv = a.sun_inv; j->sun_scale = a.sun_scale;
  j->sky = a.sky; j->sky_n = a.sky_n; j->err = a.err;
  j->shading = a.shading; j->light = a.light;
  j->probes = a.probes; j->order = const_cast<uint32_t*>(a.order); j->nprobes = a.nprobes;
  j->dirs = a.dirs; j->dinv = a.dinv; j->dir_order = a.dir_order; j->S = a.S;
  j->basis16 = a.basis16;
  j->item_begin = 0;
}

vlb_status vlb_bake_ex(vlb_ctx* ctx, const vlb_scene* scene, const float* probe_xyz, uint32_t nprobes,
                       const vlb_bake_params* p, float* out, const vlb_bake_debug* dbg) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (nprobes == 0) return VLB_OK;
  if (!out) return fail(ctx, VLB_ERR_INVALID, "null output");
  vlbk::TraceArgs a;
  vlb_status st = prepare_trace(ctx, scene, probe_xyz, nprobes, p, &a);
  if (st) return st;
  const uint32_t S = a.S, K = a.K, V = 3 * K;
  const uint64_t rays = uint64_t(nprobes) * S;
  OutBuf ob, oh, os, orad;
  if ((st = stage_out(ctx, out, size_t(nprobes) * V * 4, "bake_out", &ob))) return st;
  if (dbg) {
    if ((st = stage_out(ctx, dbg->hit_tri, rays * 4, "dbg_hit", &oh)) ||
        (st = stage_out(ctx, dbg->shadow, rays, "dbg_shadow", &os)) ||
        (st = stage_out(ctx, dbg->radiance, rays * 12, "dbg_rad", &orad)))
      return st;
    a.hit_tri = static_cast<int32_t*>(oh.dev);
    a.shadow = static_cast<uint8_t*>(os.dev);
    a.dbg_radiance = static_cast<float*>(orad.dev);
  }
  // VLB_PREC_FUSED: the lane walk with the projection in the same kernel
  // (k_trace_fused.cu), no radiance tile.  Packet walks (on request) keep the
  // packet kernel's fused mode when the directions fit at most two work items
  // per packet (large probe counts), else the tile; grid walks use the tile.
  const bool prec_fused = p->precision == VLB_PREC_FUSED;
  if (prec_fused && a.lane && !a.grid_hdr && !(p->flags & VLB_BAKE_FORCE_FUSED_KERNEL)) {
    vlbk::BakeJobDev j{};
    job_from_trace(a, &j);
    j.out = static_cast<float*>(ob.dev);
    j.chunk_rays = vlbk::fused_chunk_rays(S);
    j.chunks = (S + j.chunk_rays - 1) / j.chunk_rays;
    j.chunk_major = vlbk::fused_chunk_major(S);
    j.hit_tri = a.hit_tri; j.shadow = a.shadow; j.dbg_radiance = a.dbg_radiance;
    if (j.chunks > 1) {
      void *part, *done;
      if ((st = scratch(ctx, "bake_partial", size_t(nprobes) * j.chunks * V * 4, &part)) ||
          (st = scratch(ctx, "bake_chunk_done", size_t(nprobes) * 4, &done)))
        return st;
      VLB_CUDA(ctx, cudaMemsetAsync(done, 0, size_t(nprobes) * 4, ctx->stream));
      j.partial = static_cast<float*>(part);
      j.done = static_cast<uint32_t*>(done);
    }
    const uint64_t items = uint64_t(nprobes) * j.chunks;
    if (items >= (1ull << 32) - (1ull << 20)) return fail(ctx, VLB_ERR_INVALID, "too many probes for one bake");
    KScope k(ctx, "trace_fused_lane");
    vlbk::launch_trace_fused_lane(nullptr, j, 1, uint32_t(items), K, a.work_counter,
                                  fused_sched(class_sched(ctx, size_class(scene->ntris))),
                                  ctx->num_sms, ctx->stream);
    if (p->flags & VLB_BAKE_REF_ACCUMULATE) {
      KScope k(ctx, "probe_prefix");
      vlbk::launch_probe_prefix(static_cast<float*>(ob.dev), nprobes, V, ctx->stream);
    }
    if ((st = copy_out(ctx, ob)) || (st = copy_out(ctx, oh)) || (st = copy_out(ctx, os)) ||
        (st = copy_out(ctx, orad)))
      return st;
    return finish(ctx, ob.host || oh.host || os.host || orad.host);
  }
  bool fused = prec_fused && !a.lane && a.chunks <= 2 && !a.dbg_radiance && !a.grid_hdr;
  if (prec_fused && (p->flags & VLB_BAKE_FORCE_FUSED_KERNEL)) {
    if (a.dbg_radiance) return fail(ctx, VLB_ERR_UNSUPPORTED, "the fused kernel keeps no per-ray radiance");
    fused = true;
  }
  if (prec_fused && !fused) vlbk::plan_trace(a, ctx->num_sms, false);
  if (fused) {
    a.out = static_cast<float*>(ob.dev);
    if (a.chunks > 1) {
      void *part, *done;
      const size_t groups = (size_t(nprobes) + 31) / 32;
      if ((st = scratch(ctx, "bake_partial", size_t(nprobes) * a.chunks * V * 4, &part)) ||
          (st = scratch(ctx, "bake_group_done", groups * 4, &done)))
        return st;
      VLB_CUDA(ctx, cudaMemsetAsync(done, 0, groups * 4, ctx->stream));
      a.partial = static_cast<float*>(part);
      a.group_done = static_cast<uint32_t*>(done);
    }
    KScope k(ctx, "trace_fused");
    vlbk::launch_trace_fused(a, ctx->num_sms, ctx->stream);
  } else {
    const bool bf16 = p->precision == VLB_PREC_MIXED || p->precision == VLB_PREC_BF16;
    const bool split = p->precision == VLB_PREC_MIXED;
    if (split && (st = dirset_split_basis(ctx, p->dirs))) return st;
    void* tile;
    if ((st = scratch(ctx, "bake_tile", rays * 3 * (bf16 && !split ? 2 : 4), &tile))) return st;
    if (bf16) a.radiance_bf16 = static_cast<uint16_t*>(tile);
    else a.radiance = static_cast<float*>(tile);
    a.bf16_split = split ? 1 : 0;
    {
      KScope k(ctx, "trace_tile");
      vlbk::launch_trace_tile(a, ctx->num_sms, ctx->stream);
    }
    if (bf16) {
      if ((st = project_bf16(ctx, a.radiance_bf16, nprobes, p->dirs, K, static_cast<float*>(ob.dev), split)))
        return st;
    } else if ((st = project_f32(ctx, a.radiance, nprobes, p->dirs, K, static_cast<float*>(ob.dev)))) {
      return st;
    }
  }
  if (p->flags & VLB_BAKE_REF_ACCUMULATE) {
    KScope k(ctx, "probe_prefix");
    vlbk::launch_probe_prefix(static_cast<float*>(ob.dev), nprobes, V, ctx->stream);
  }
  if ((st = copy_out(ctx, ob)) || (st = copy_out(ctx, oh)) || (st = copy_out(ctx, os)) || (st = copy_out(ctx, orad)))
    return st;
  return finish(ctx, ob.host || oh.host || os.host || orad.host);
}

vlb_status vlb_bake(vlb_ctx* ctx, const vlb_scene* scene, const float* probe_xyz, uint32_t nprobes,
                    const vlb_bake_params* params, float* out) {
  return vlb_bake_ex(ctx, scene, probe_xyz, nprobes, params, out, nullptr);
}

vlb_status vlb_bake_async(vlb_ctx* ctx, const vlb_scene* scene, const float* probe_xyz, uint32_t nprobes,
                          const vlb_bake_params* params, float* out, void* done_event) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (nprobes && (!is_device_ptr(probe_xyz) || !is_device_ptr(out)))
    return fail(ctx, VLB_ERR_INVALID, "vlb_bake_async needs device probes and a device output");
  const vlb_status st = vlb_bake_ex(ctx, scene, probe_xyz, nprobes, params, out, nullptr);
  if (st) return st;
  if (done_event) VLB_CUDA(ctx, cudaEventRecord(static_cast<cudaEvent_t>(done_event), ctx->stream));
  return VLB_OK;
}

vlb_status vlb_bake_trace_stats(vlb_ctx* ctx, const vlb_scene* scene, const float* probe_xyz, uint32_t nprobes,
                                const vlb_bake_params* p, uint64_t out[6]) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (!out || nprobes == 0) return fail(ctx, VLB_ERR_INVALID, "no probes or no output");
  vlbk::TraceArgs a;
  vlb_status st = prepare_trace(ctx, scene, probe_xyz, nprobes, p, &a);
  if (st) return st;
  void *tile, *cnt;
  if ((st = scratch(ctx, "bake_tile", size_t(nprobes) * a.S * 12, &tile)) ||
      (st = scratch(ctx, "trace_counters", 64, &cnt)))
    return st;
  VLB_CUDA(ctx, cudaMemsetAsync(cnt, 0, 64, ctx->stream));
  a.radiance = static_cast<float*>(tile);
  a.counters = static_cast<unsigned long long*>(cnt);
  {
    KScope k(ctx, "trace_tile_counted");
    vlbk::launch_trace_tile(a, ctx->num_sms, ctx->stream);
  }
  if ((st = finish(ctx, true))) return st;
  unsigned long long h[4];
  VLB_CUDA(ctx, cudaMemcpy(h, cnt, sizeof h, cudaMemcpyDeviceToHost));
  out[0] = uint64_t(nprobes) * a.S;
  out[1] = h[2];
  out[2] = h[0];
  out[3] = h[1];
  out[4] = h[3];
  out[5] = a.lane && a.wnodes && !a.grid_hdr ? 96 : 64;  // the tile lane walk walks the wide tree
  return VLB_OK;
}

// ---- batched bakes ---------------------------------------------------------------------------
namespace {

struct BatchJob {
  uint32_t idx;               // caller's job index
  const vlb_bake_params* p;   // effective parameters
  double sun_len;
  uint32_t nprobes, S, group;
  uint64_t row0;              // first row of the concatenated output (direction sets contiguous)
  double cost;
};

struct BatchGroup {
  const vlb_dirset* dirs;
  uint64_t row0, rows;
  size_t tile_off;            // bytes into the batch tile (256-byte aligned)
};

struct BatchPlan {
  std::vector<BatchJob> jobs;     // non-empty jobs, caller order
  std::vector<BatchGroup> groups;
  uint64_t rows = 0;
  size_t tile_bytes = 0, host_probe_bytes = 0;
  uint32_t K = 0;
  uint32_t max_probes = 0;  // largest job
  bool bf16 = false;
  bool split = false;         // VLB_PREC_MIXED: BF16 hi/lo pairs
  bool fused = false;         // VLB_PREC_FUSED: the fused lane walk, no tile
  size_t partial_floats = 0;  // fused: chunk partials of all jobs
};

// Device buffers of one batch (context scratch, allocated before any launch
// so that the launch sequence can be captured).
struct BatchBufs {
  float* probes;       // packed host-side probes
  uint32_t* order;     // rows
  uint32_t* sort;      // 4 x rows
  uint8_t* tile;
  float* out;          // rows x V
  float* partial;      // fused: chunk partials
  uint32_t* done;      // fused: rows chunk tickets
  uint8_t* meta;       // job table + scatter arrays
  uint32_t* counter;
  size_t table_bytes, dst_off, p0_off, np_off;
  uint32_t ndev_out;   // jobs whose output is device memory (scattered by a kernel)
};

}  // namespace

static vlb_status batch_plan(vlb_ctx* ctx, const vlb_bake_job* jobs, uint32_t njobs, const vlb_bake_params* params,
                             BatchPlan* pl) {
  if (!params) return fail(ctx, VLB_ERR_INVALID, "null batch params");
  if (!jobs && njobs) return fail(ctx, VLB_ERR_INVALID, "null job array");
  if (params->lmax != 2 && params->lmax != 3) return fail(ctx, VLB_ERR_INVALID, "lmax must be 2 or 3 (got %u)", params->lmax);
  if (params->precision > VLB_PREC_BF16) return fail(ctx, VLB_ERR_INVALID, "precision %u", params->precision);
  pl->K = k_of(params->lmax);
  pl->bf16 = params->precision == VLB_PREC_MIXED || params->precision == VLB_PREC_BF16;
  pl->split = params->precision == VLB_PREC_MIXED;
  pl->fused = params->precision == VLB_PREC_FUSED;
  for (uint32_t i = 0; i < njobs; ++i) {
    const vlb_bake_job& j = jobs[i];
    const vlb_bake_params* p = j.params ? j.params : params;
    BatchJob b{};
    vlb_status st = check_params(ctx, j.scene, p, &b.sun_len);
    if (st) return fail(ctx, st, "job %u: %s", i, ctx->err.c_str());
    if (p->lmax != params->lmax || p->precision != params->precision || p->shading != params->shading)
      return fail(ctx, VLB_ERR_INVALID, "job %u: lmax, precision and shading must equal the batch's", i);
    if (j.nprobes == 0) continue;
    if (!j.probe_xyz || !j.out) return fail(ctx, VLB_ERR_INVALID, "job %u: null probes or output", i);
    b.idx = i; b.p = p; b.nprobes = j.nprobes; b.S = p->dirs->n;
    if (pl->fused) {
      const uint32_t D = vlbk::fused_chunk_rays(b.S), C = (b.S + D - 1) / D;
      if (C > 1) pl->partial_floats += size_t(j.nprobes) * C * 3 * pl->K;
    }
    pl->max_probes = std::max(pl->max_probes, j.nprobes);
    b.cost = double(j.nprobes) * b.S * std::log2(double(j.scene->ntris) + 2.0);
    uint32_t g = 0;
    while (g < pl->groups.size() && pl->groups[g].dirs != p->dirs) ++g;
    if (g == pl->groups.size()) pl->groups.push_back({p->dirs, 0, 0, 0});
    b.group = g;
    pl->groups[g].rows += j.nprobes;
    if (!is_device_ptr(j.probe_xyz)) pl->host_probe_bytes += (size_t(j.nprobes) * 12 + 15) / 16 * 16;
    pl->jobs.push_back(b);
  }
  const size_t esz = pl->bf16 && !pl->split ? 2 : 4;  // bytes a sample (hi/lo pairs: 4)
  for (auto& g : pl->groups) {
    g.row0 = pl->rows;
    pl->rows += g.rows;
    g.tile_off = pl->tile_bytes;
    if (!pl->fused) pl->tile_bytes += (size_t(g.rows) * 3 * g.dirs->n * esz + 255) / 256 * 256;
    g.rows = 0;  // reused below as the running row
  }
  for (auto& b : pl->jobs) {
    auto& g = pl->groups[b.group];
    b.row0 = g.row0 + g.rows;
    g.rows += b.nprobes;
  }
  if (pl->rows > 0xFFFFFFFFull / 16) return fail(ctx, VLB_ERR_INVALID, "batch too large (%llu probes)",
                                                   (unsigned long long)pl->rows);
  return VLB_OK;
}

// The device work of a batch on ctx->stream (capturable: no allocation, no
// synchronisation).
static vlb_status batch_enqueue(vlb_ctx* ctx, const BatchPlan& pl, const BatchBufs& bb, uint32_t ntable,
                                uint32_t total_rays, uint32_t chunk, const vlbk::FusedSched& fs) {
  const uint32_t V = 3 * pl.K;
  const auto* table = reinterpret_cast<const vlbk::BakeJobDev*>(bb.meta);
  VLB_CUDA(ctx, cudaMemsetAsync(bb.counter, 0, 4, ctx->stream));
  if (pl.fused) VLB_CUDA(ctx, cudaMemsetAsync(bb.done, 0, pl.rows * 4, ctx->stream));
  {
    KScope k(ctx, "probe_order_batch");
    vlbk::launch_probe_order_batch(table, ntable, ctx->stream);
  }
  if (pl.fused) {
    KScope k(ctx, "trace_fused_batch");
    vlbk::launch_trace_fused_lane(table, ctx->batch_table[0], ntable, total_rays, pl.K, bb.counter, fs,
                                  ctx->num_sms, ctx->stream);
  } else {
    KScope k(ctx, "trace_batch");
    vlbk::launch_trace_batch(table, ntable, total_rays, chunk, bb.counter,
                             ctx->batch_table[0].shading == VLB_SHADE_REF_PHONG, ctx->num_sms, ctx->stream);
  }
  for (const auto& g : pl.groups) {
    if (pl.fused) break;  // the fused walk wrote the projected rows
    float* out = bb.out + g.row0 * V;
    const uint32_t n = uint32_t(g.rows);
    if (pl.bf16) {
      vlb_status st = project_bf16(ctx, reinterpret_cast<const uint16_t*>(bb.tile + g.tile_off), n, g.dirs, pl.K, out,
                                   pl.split, "batch_project_partial");
      if (st) return st;
    } else {
      vlb_status st = project_f32(ctx, reinterpret_cast<const float*>(bb.tile + g.tile_off), n, g.dirs, pl.K, out,
                                  "batch_project_partial");
      if (st) return st;
    }
  }
  if (bb.ndev_out) {
    KScope k(ctx, "scatter_rows");
    vlbk::launch_scatter_rows(bb.out, reinterpret_cast<float* const*>(bb.meta + bb.dst_off),
                              reinterpret_cast<const uint32_t*>(bb.meta + bb.p0_off),
                              reinterpret_cast<const uint32_t*>(bb.meta + bb.np_off), bb.ndev_out, pl.K, ctx->stream);
  }
  return VLB_OK;
}

}  // extern "C"

// Enqueues a batch on ctx->stream and returns without waiting.  Host
// outputs are copied with cudaMemcpyAsync (asynchronous only for pinned
// memory); *host_out tells whether there were any.  ext (optional, njobs
// entries) adds kept-hit outputs and relight inputs per job.
vlb_status vlbh::batch_launch(vlb_ctx* ctx, const vlb_bake_job* jobs, const vlbh::JobExt* ext, uint32_t njobs,
                              const vlb_bake_params* params, const vlb_batch_schedule& sc, bool* host_out_any) {
  *host_out_any = false;
  BatchPlan pl;
  vlb_status st = batch_plan(ctx, jobs, njobs, params, &pl);
  if (st) return st;
  if (pl.jobs.empty()) return VLB_OK;
  const uint32_t K = pl.K, V = 3 * K;
  const uint32_t ntable = uint32_t(pl.jobs.size());
  // job table order: costliest first (or caller order)
  std::vector<uint32_t> ord(ntable);
  for (uint32_t i = 0; i < ntable; ++i) ord[i] = i;
  if (sc.cost_order)
    std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return pl.jobs[a].cost > pl.jobs[b].cost; });
  uint32_t ndev_out = 0;
  for (const auto& b : pl.jobs) ndev_out += is_device_ptr(jobs[b.idx].out) ? 1 : 0;
  BatchBufs bb{};
  bb.table_bytes = (size_t(ntable) * sizeof(vlbk::BakeJobDev) + 255) / 256 * 256;
  bb.dst_off = bb.table_bytes;
  bb.p0_off = bb.dst_off + size_t(ndev_out) * 8;
  bb.np_off = bb.p0_off + size_t(ndev_out) * 4;
  bb.ndev_out = ndev_out;
  const size_t meta_bytes = bb.np_off + size_t(ndev_out) * 4;
  void *probes = nullptr, *order, *sort, *tile = nullptr, *out, *meta, *counter, *part = nullptr, *done = nullptr;
  if ((pl.host_probe_bytes && (st = scratch(ctx, "batch_probes", pl.host_probe_bytes, &probes))) ||
      (st = scratch(ctx, "batch_order", pl.rows * 4, &order)) ||
      (st = scratch(ctx, "batch_sort", pl.rows * 16, &sort)) ||
      (pl.tile_bytes && (st = scratch(ctx, "batch_tile", pl.tile_bytes, &tile))) ||
      (st = scratch(ctx, "batch_out", pl.rows * V * 4, &out)) ||
      (st = scratch(ctx, "batch_meta", meta_bytes, &meta)) ||
      (st = scratch(ctx, "batch_counter", 256, &counter)) ||
      (pl.partial_floats && (st = scratch(ctx, "batch_partial", pl.partial_floats * 4, &part))) ||
      (pl.fused && (st = scratch(ctx, "batch_done", pl.rows * 4, &done))))
    return st;
  bb.partial = static_cast<float*>(part); bb.done = static_cast<uint32_t*>(done);
  bb.probes = static_cast<float*>(probes); bb.order = static_cast<uint32_t*>(order);
  bb.sort = static_cast<uint32_t*>(sort); bb.tile = static_cast<uint8_t*>(tile); bb.out = static_cast<float*>(out);
  bb.meta = static_cast<uint8_t*>(meta); bb.counter = static_cast<uint32_t*>(counter);

  // stage host probes, build the job table
  const size_t esz = pl.bf16 && !pl.split ? 2 : 4;
  uint64_t warp_rays = 0;
  for (const auto& b : pl.jobs) warp_rays += (uint64_t(b.nprobes) + 31) / 32 * b.S;
  // rays per lane per chunk (a warp takes 32 x that many rays at a time):
  // at least ~16 chunks per resident warp, at most 8 rays per lane
  uint32_t dpw = sc.dirs_per_item;
  if (!dpw) {
    uint64_t rays = 0;
    for (const auto& b : pl.jobs) rays += (uint64_t(b.nprobes) + 31) / 32 * 32 * b.S;
    const uint64_t target = 16ull * 32 * 32 * uint64_t(ctx->num_sms);
    dpw = uint32_t(std::min<uint64_t>(8, std::max<uint64_t>(1, rays / target)));
  }
  const uint32_t chunk = 32 * dpw;
  if (pl.split)  // the split basis is built before anything is enqueued (or captured)
    for (const auto& g : pl.groups)
      if ((st = dirset_split_basis(ctx, g.dirs))) return st;
  auto& table = ctx->batch_table;
  table.assign(ntable, vlbk::BakeJobDev{});
  size_t poff = 0, part_off = 0;
  uint64_t items = 0;
  for (uint32_t t = 0; t < ntable; ++t) {
    const BatchJob& b = pl.jobs[ord[t]];
    const vlb_bake_job& j = jobs[b.idx];
    const vlb_bake_params* p = b.p;
    const BatchGroup& g = pl.groups[b.group];
    vlbk::BakeJobDev& d = table[t];
    d.nodes = j.scene->nodes; d.tris = j.scene->tris; d.albedo = j.scene->albedo; d.ntris = j.scene->ntris;
    d.wnodes = j.scene->wnodes;
    d.nwide = j.scene->nwide;
    d.tmin = p->tmin; d.tmax = p->tmax; d.bias = p->shadow_bias;
    d.sun = make_float3(float(p->sun_dir[0] / b.sun_len), float(p->sun_dir[1] / b.sun_len),
                        float(p->sun_dir[2] / b.sun_len));
    d.sun_inv =
        make_float3(vlbk::host_safe_inv(d.sun.x), vlbk::host_safe_inv(d.sun.y), vlbk::host_safe_inv(d.sun.z));
    d.sun_scale = float(double(p->sun_intensity) / kPi);
    d.sky = p->sky ? p->sky->d_texels : nullptr; d.sky_n = p->sky ? p->sky->n : 0;
    d.shading = p->shading;
    d.light = make_float3(p->light_pos[0], p->light_pos[1], p->light_pos[2]);
    d.err = ctx->d_err;
    if (is_device_ptr(j.probe_xyz)) {
      d.probes = j.probe_xyz;
    } else {
      float* dst = reinterpret_cast<float*>(static_cast<uint8_t*>(probes) + poff);
      VLB_CUDA(ctx, cudaMemcpyAsync(dst, j.probe_xyz, size_t(b.nprobes) * 12, cudaMemcpyHostToDevice, ctx->stream));
      ctx->host_inputs_pending = true;
      d.probes = dst;
      poff += (size_t(b.nprobes) * 12 + 15) / 16 * 16;
    }
    d.order = bb.order + b.row0;
    d.nprobes = b.nprobes;
    d.dirs = p->dirs->d_dirs; d.dinv = p->dirs->d_dinv; d.dir_order = p->dirs->d_order; d.S = b.S;
    if (pl.fused) {
      d.basis16 = p->dirs->d_basis16;
      d.out = bb.out + b.row0 * V;
      d.chunk_rays = vlbk::fused_chunk_rays(b.S);
      d.chunks = (b.S + d.chunk_rays - 1) / d.chunk_rays;
      d.chunk_major = vlbk::fused_chunk_major(b.S);
      if (d.chunks > 1) {
        d.partial = bb.partial + part_off;
        part_off += size_t(b.nprobes) * d.chunks * V;
      }
      d.done = bb.done + b.row0;
      d.item_begin = uint32_t(items);
      items += uint64_t(b.nprobes) * d.chunks;
    } else {
      uint8_t* rad = bb.tile + g.tile_off + (b.row0 - g.row0) * 3 * b.S * esz;
      d.bf16_split = pl.split ? 1 : 0;
      if (pl.bf16) d.radiance_bf16 = reinterpret_cast<uint16_t*>(rad);
      else d.radiance = reinterpret_cast<float*>(rad);
      d.ray_begin = uint32_t(items);
      items += ((uint64_t(b.nprobes) + 31) / 32 * 32 * b.S + chunk - 1) / chunk * chunk;
    }
    for (int a = 0; a < 6; ++a) d.bounds[a] = j.scene->bounds[a];
    d.sort_scratch = bb.sort + 4 * b.row0;
    if (ext) { d.hits_out = ext[b.idx].hits_out; d.hits_in = ext[b.idx].hits_in; }
  }
  if (items >= (1ull << 31))
    return fail(ctx, VLB_ERR_INVALID, pl.fused ? "batch has 2^31 work items or more; split it"
                                               : "batch has 2^31 rays or more; split it");
  auto& meta_h = ctx->batch_meta;
  meta_h.assign(meta_bytes, 0);
  std::memcpy(meta_h.data(), table.data(), table.size() * sizeof(vlbk::BakeJobDev));
  {
    uint32_t k = 0;
    for (const auto& b : pl.jobs) {
      float* o = jobs[b.idx].out;
      if (!is_device_ptr(o)) continue;
      const uint32_t p0 = uint32_t(b.row0), np = b.nprobes;
      std::memcpy(meta_h.data() + bb.dst_off + 8 * k, &o, 8);
      std::memcpy(meta_h.data() + bb.p0_off + 4 * k, &p0, 4);
      std::memcpy(meta_h.data() + bb.np_off + 4 * k, &np, 4);
      ++k;
    }
  }
  VLB_CUDA(ctx, cudaMemcpyAsync(meta, meta_h.data(), meta_bytes, cudaMemcpyHostToDevice, ctx->stream));

  // shape key: everything the captured launches bake in as parameters
  std::vector<uint64_t> key = {ntable, uint64_t(items), dpw, pl.bf16 + 2u * pl.split, K, ndev_out, pl.max_probes,
                               uint64_t(uintptr_t(tile)), uint64_t(uintptr_t(out)), uint64_t(uintptr_t(meta)),
                               uint64_t(uintptr_t(counter)), uint64_t(ctx->num_sms), pl.fused,
                               uint64_t(uintptr_t(part)), uint64_t(uintptr_t(done)), pl.rows, sc.ctas_per_sm,
                               sc.node_steps, sc.refill_idle};
  if (pl.fused && ntable == 1) {  // one job goes to the kernel by value: its fields are part of the shape
    const auto* w = reinterpret_cast<const uint64_t*>(table.data());
    key.insert(key.end(), w, w + sizeof(vlbk::BakeJobDev) / 8);
  }
  for (const auto& g : pl.groups) {
    key.push_back(uint64_t(uintptr_t(g.dirs)));
    key.push_back(g.row0); key.push_back(g.rows); key.push_back(g.tile_off);
  }
  const bool same = ctx->batch_key == key;
  if (!same) {
    if (ctx->batch_exec) { cudaGraphExecDestroy(ctx->batch_exec); ctx->batch_exec = nullptr; }
    ctx->batch_key = key;
  }
  if (sc.graph && same) {
    if (!ctx->batch_exec) {
      const bool prof = ctx->profiling;
      const uint64_t l0 = ctx->launches;
      ctx->profiling = false;
      cudaGraph_t g = nullptr;
      VLB_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      st = batch_enqueue(ctx, pl, bb, ntable, uint32_t(items), chunk, fused_sched(sc));
      const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
      ctx->profiling = prof;
      ctx->batch_graph_kernels = uint32_t(ctx->launches - l0);
      ctx->launches = l0;
      if (st) { if (g) cudaGraphDestroy(g); return st; }
      if (e != cudaSuccess) { cudaGetLastError(); return cuda_fail(ctx, e, "batch graph capture"); }
      const cudaError_t ei = cudaGraphInstantiate(&ctx->batch_exec, g, 0ull);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) { ctx->batch_exec = nullptr; return cuda_fail(ctx, ei, "batch graph instantiate"); }
    }
    KScope k(ctx, "bake_batch_graph", int(ctx->batch_graph_kernels));
    VLB_CUDA(ctx, cudaGraphLaunch(ctx->batch_exec, ctx->stream));
  } else if ((st = batch_enqueue(ctx, pl, bb, ntable, uint32_t(items), chunk, fused_sched(sc)))) {
    return st;
  }
  for (const auto& b : pl.jobs) {
    float* o = jobs[b.idx].out;
    if (is_device_ptr(o)) continue;
    *host_out_any = true;
    VLB_CUDA(ctx, cudaMemcpyAsync(o, bb.out + b.row0 * V, size_t(b.nprobes) * V * 4, cudaMemcpyDeviceToHost,
                                  ctx->stream));
  }
  return VLB_OK;
}

extern "C" {

static vlb_status batch_run(vlb_ctx* ctx, const vlb_bake_job* jobs, uint32_t njobs, const vlb_bake_params* params,
                            const vlb_batch_schedule& sc) {
  bool host_out = false;
  const vlb_status st = vlbh::batch_launch(ctx, jobs, nullptr, njobs, params, sc, &host_out);
  if (st) return st;
  return finish(ctx, host_out);
}

}  // extern "C"

vlb_status vlbh::ctx_finish(vlb_ctx* ctx, bool sync) { return finish(ctx, sync); }

vlb_status vlbh::ctx_fail(vlb_ctx* ctx, vlb_status s, const char* msg) { return fail(ctx, s, "%s", msg); }

extern "C" {

vlb_status vlb_bake_batch(vlb_ctx* ctx, const vlb_bake_job* jobs, uint32_t njobs, const vlb_bake_params* params,
                          const vlb_batch_schedule* sched) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  vlb_batch_schedule sc = sched ? *sched : class_sched(ctx, batch_class(jobs, njobs));
  if (sc.dirs_per_item > 64) return fail(ctx, VLB_ERR_INVALID, "dirs_per_item %u > 64", sc.dirs_per_item);
  if (sc.ctas_per_sm && (sc.ctas_per_sm < 7 || sc.ctas_per_sm > 9))
    return fail(ctx, VLB_ERR_INVALID, "ctas_per_sm %u: 7, 8 or 9", sc.ctas_per_sm);
  if (sc.node_steps > 16 || sc.refill_idle > 32)
    return fail(ctx, VLB_ERR_INVALID, "node_steps %u (<= 16) or refill_idle %u (<= 32)", sc.node_steps,
                sc.refill_idle);
  return batch_run(ctx, jobs, njobs, params, sc);
}

vlb_status vlb_batch_autotune(vlb_ctx* ctx, const vlb_bake_job* jobs, uint32_t njobs, const vlb_bake_params* params,
                              uint32_t reps, vlb_batch_schedule* best, float* best_ms) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (!params) return fail(ctx, VLB_ERR_INVALID, "null batch params");
  if (reps == 0) reps = 1;
  cudaEvent_t e0, e1;
  VLB_CUDA(ctx, cudaEventCreate(&e0));
  VLB_CUDA(ctx, cudaEventCreate(&e1));
  // mean ms per batch of one schedule (after one warm-up run), or < 0 on error
  vlb_status st = VLB_OK;
  auto time_one = [&](const vlb_batch_schedule& sc) -> float {
    if ((st = batch_run(ctx, jobs, njobs, params, sc))) return -1.f;
    cudaEventRecord(e0, ctx->stream);
    for (uint32_t r = 0; r < reps && !st; ++r) st = batch_run(ctx, jobs, njobs, params, sc);
    cudaEventRecord(e1, ctx->stream);
    if (st) return -1.f;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      st = cuda_fail(ctx, cudaGetLastError(), "autotune timing");
      return -1.f;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms / float(reps);
  };
  vlb_batch_schedule win{0, 1, 1, 0, 0, 0};
  float win_ms = -1.f;
  std::vector<vlb_tune_trial> log;
  auto trial = [&](const vlb_batch_schedule& c) {
    const float ms = time_one(c);
    if (ms >= 0.f) log.push_back({c, ms});
    if (ms >= 0.f && (win_ms < 0.f || ms < win_ms)) { win_ms = ms; win = c; }
  };
  if (params->precision == VLB_PREC_FUSED) {
    // one knob at a time from the default, each kept at its fastest value
    trial(vlb_batch_schedule{0, 1, 0, 8, 6, 32});
    auto sweep = [&](uint32_t vlb_batch_schedule::*knob, std::initializer_list<uint32_t> vals) {
      const vlb_batch_schedule base = win;
      for (uint32_t v : vals) {
        if (st) return;
        if (base.*knob == v) continue;
        vlb_batch_schedule c = base;
        c.*knob = v;
        trial(c);
      }
    };
    sweep(&vlb_batch_schedule::ctas_per_sm, {7, 9});
    sweep(&vlb_batch_schedule::node_steps, {2, 4, 8, 12, 16});
    sweep(&vlb_batch_schedule::refill_idle, {8, 16, 24});
    sweep(&vlb_batch_schedule::cost_order, {0});
  } else {
    const uint32_t dpws[] = {0, 1, 2, 4, 8, 16};
    for (uint32_t order : {1u, 0u})
      for (uint32_t dpw : dpws) {
        if (st) break;
        trial(vlb_batch_schedule{dpw, order, 0, 0, 0, 0});
      }
  }
  win.graph = 1;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  const uint32_t cls = batch_class(jobs, njobs);
  ctx->tuned[cls] = win;
  ctx->tuned_set[cls] = true;
  ctx->tune_log = std::move(log);
  ctx->tune_class = cls;
  if (best) *best = win;
  if (best_ms) *best_ms = win_ms;
  return finish(ctx, true);
}

vlb_status vlb_batch_tune_log(const vlb_ctx* ctx, vlb_tune_trial* out, uint32_t cap, uint32_t* n,
                              uint32_t* size_class_out) {
  if (!ctx || !n) return VLB_ERR_INVALID;
  const uint32_t m = uint32_t(ctx->tune_log.size());
  for (uint32_t i = 0; out && i < m && i < cap; ++i) out[i] = ctx->tune_log[i];
  *n = m;
  if (size_class_out) *size_class_out = ctx->tune_class;
  return VLB_OK;
}

// ---- evaluating a baked grid ------------------------------------------------------------------
vlb_status vlb_probe_eval(vlb_ctx* ctx, const vlb_scene* scene, const float* coeffs, uint32_t lmax,
                          const vlb_probe_grid* g, const float* points, const float* normals, uint32_t n,
                          float shadow_bias, float* out_rgb, uint8_t* vis_mask) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (lmax != 2 && lmax != 3) return fail(ctx, VLB_ERR_INVALID, "lmax must be 2 or 3 (got %u)", lmax);
  if (!g) return fail(ctx, VLB_ERR_INVALID, "null grid");
  if (scene && scene->ctx != ctx) return fail(ctx, VLB_ERR_INVALID, "scene belongs to another context");
  uint64_t nprobes = 1;
  for (int a = 0; a < 3; ++a) {
    if (g->counts[a] == 0) return fail(ctx, VLB_ERR_INVALID, "grid counts must be positive");
    if (g->counts[a] > 1 && !(g->step[a] > 0.f && std::isfinite(g->step[a])))
      return fail(ctx, VLB_ERR_INVALID, "grid step must be positive and finite on axes with more than one probe");
    nprobes *= g->counts[a];
  }
  if (nprobes > 0xFFFFFFFFull) return fail(ctx, VLB_ERR_INVALID, "grid too large");
  if (n == 0) return VLB_OK;
  if (!coeffs || !points || !normals || !out_rgb) return fail(ctx, VLB_ERR_INVALID, "null array");
  const uint32_t K = k_of(lmax);
  vlb_status st;
  const void *dc, *dp, *dn;
  OutBuf ob, ov;
  if ((st = stage_in(ctx, coeffs, nprobes * K * 12, "eval_coeffs", &dc)) ||
      (st = stage_in(ctx, points, size_t(n) * 12, "eval_points", &dp)) ||
      (st = stage_in(ctx, normals, size_t(n) * 12, "eval_normals", &dn)) ||
      (st = stage_out(ctx, out_rgb, size_t(n) * 12, "eval_out", &ob)) ||
      (st = stage_out(ctx, vis_mask, n, "eval_vis", &ov)))
    return st;
  vlbk::ProbeEvalArgs a{};
  if (scene && scene->ntris) { a.nodes = scene->nodes; a.tris = scene->tris; a.ntris = scene->ntris; }
  a.coeffs = static_cast<const float*>(dc);
  for (int c = 0; c < 3; ++c) { a.org[c] = g->origin[c]; a.step[c] = g->step[c]; a.counts[c] = g->counts[c]; }
  a.points = static_cast<const float*>(dp);
  a.normals = static_cast<const float*>(dn);
  a.n = n;
  a.bias = shadow_bias;
  a.out = static_cast<float*>(ob.dev);
  a.vis = static_cast<uint8_t*>(ov.dev);
  a.err = ctx->d_err;
  {
    KScope k(ctx, "probe_eval");
    vlbk::launch_probe_eval(a, lmax, ctx->stream);
  }
  if ((st = copy_out(ctx, ob)) || (st = copy_out(ctx, ov))) return st;
  return finish(ctx, ob.host || ov.host);
}

vlb_status vlb_sh_eval_dirs(vlb_ctx* ctx, const float* coeffs, uint32_t lmax, const float* dirs, uint32_t n,
                            float* out_rgb) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (lmax != 2 && lmax != 3) return fail(ctx, VLB_ERR_INVALID, "lmax must be 2 or 3 (got %u)", lmax);
  if (n == 0) return VLB_OK;
  if (!coeffs || !dirs || !out_rgb) return fail(ctx, VLB_ERR_INVALID, "null array");
  vlb_status st;
  const void *dc, *dd;
  OutBuf ob;
  if ((st = stage_in(ctx, coeffs, size_t(k_of(lmax)) * 12, "evald_coeffs", &dc)) ||
      (st = stage_in(ctx, dirs, size_t(n) * 12, "evald_dirs", &dd)) ||
      (st = stage_out(ctx, out_rgb, size_t(n) * 12, "evald_out", &ob)))
    return st;
  {
    KScope k(ctx, "sh_eval_dirs");
    vlbk::launch_sh_eval_dirs(static_cast<const float*>(dc), lmax, static_cast<const float*>(dd), n,
                              static_cast<float*>(ob.dev), ctx->stream);
  }
  if ((st = copy_out(ctx, ob))) return st;
  return finish(ctx, ob.host);
}

// ---- debug env-map images -----------------------------------------------------------------
vlb_status vlb_encode_rgba8(vlb_ctx* ctx, const float* rgb, uint32_t n, float scale, uint32_t srgb, uint8_t* rgba) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (n == 0) return VLB_OK;
  if (!rgb || !rgba) return fail(ctx, VLB_ERR_INVALID, "null array");
  vlb_status st;
  const void* d;
  OutBuf ob;
  if ((st = stage_in(ctx, rgb, size_t(n) * 12, "enc_in", &d)) ||
      (st = stage_out(ctx, rgba, size_t(n) * 4, "enc_out", &ob)))
    return st;
  {
    KScope k(ctx, "encode_rgba8");
    vlbk::launch_encode_rgba8(static_cast<const float*>(d), n, scale, srgb ? 1u : 0u,
                              static_cast<uint8_t*>(ob.dev), ctx->num_sms, ctx->stream);
  }
  if ((st = copy_out(ctx, ob))) return st;
  return finish(ctx, ob.host);
}

vlb_status vlb_render_envmap(vlb_ctx* ctx, const vlb_scene* scene, const float probe_xyz[3],
                             const vlb_bake_params* p, uint32_t w, uint32_t h, uint8_t* rgba) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (!p || !p->dirs || !probe_xyz || !rgba) return fail(ctx, VLB_ERR_INVALID, "null argument");
  if (uint64_t(w) * h != p->dirs->n || w == 0)
    return fail(ctx, VLB_ERR_INVALID, "params->dirs must hold w*h = %llu samples (it holds %u)",
                (unsigned long long)(uint64_t(w) * h), p->dirs->n);
  if (p->precision == VLB_PREC_FUSED)
    return fail(ctx, VLB_ERR_UNSUPPORTED, "the fused schedule keeps no per-ray radiance");
  const size_t S = p->dirs->n;
  void *rad, *sh;
  vlb_status st;
  if ((st = scratch(ctx, "env_rad", S * 12, &rad)) || (st = scratch(ctx, "env_sh", 16 * 12, &sh))) return st;
  float probe[3] = {probe_xyz[0], probe_xyz[1], probe_xyz[2]};
  const void* dprobe;
  if ((st = stage_in(ctx, probe, 12, "env_probe", &dprobe))) return st;
  vlb_bake_debug dbg{nullptr, nullptr, static_cast<float*>(rad)};
  if ((st = vlb_bake_ex(ctx, scene, static_cast<const float*>(dprobe), 1, p, static_cast<float*>(sh), &dbg)))
    return st;
  return vlb_encode_rgba8(ctx, static_cast<const float*>(rad), uint32_t(S), 1.0f, 1u, rgba);
}

// ---- projection / reconstruction --------------------------------------------------------
vlb_status vlb_project(vlb_ctx* ctx, const void* radiance, vlb_dtype dtype, uint32_t nprobes, const vlb_dirset* dirs,
                       uint32_t lmax, float* out) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (!dirs || dirs->ctx != ctx) return fail(ctx, VLB_ERR_INVALID, "direction set missing or from another context");
  if (lmax != 2 && lmax != 3) return fail(ctx, VLB_ERR_INVALID, "lmax must be 2 or 3 (got %u)", lmax);
  if (dtype != VLB_DTYPE_F32 && dtype != VLB_DTYPE_BF16 && dtype != VLB_DTYPE_BF16_SPLIT)
    return fail(ctx, VLB_ERR_INVALID, "dtype %d", dtype);
  if (nprobes == 0) return VLB_OK;
  if (!radiance || !out) return fail(ctx, VLB_ERR_INVALID, "null radiance or output");
  const uint32_t S = dirs->n, K = k_of(lmax);
  const size_t eb = dtype == VLB_DTYPE_BF16 ? 2 : 4;  // bytes a sample (hi/lo pairs: 4)
  const bool split = dtype == VLB_DTYPE_BF16_SPLIT;
  vlb_status st;
  if (split && (st = dirset_split_basis(ctx, dirs))) return st;
  const void* drad;
  if ((st = stage_in(ctx, radiance, size_t(nprobes) * 3 * S * eb, "proj_in", &drad))) return st;
  OutBuf ob;
  if ((st = stage_out(ctx, out, size_t(nprobes) * K * 12, "proj_out", &ob))) return st;
  if (dtype == VLB_DTYPE_F32) {
    if ((st = project_f32(ctx, static_cast<const float*>(drad), nprobes, dirs, K, static_cast<float*>(ob.dev))))
      return st;
  } else if ((st = project_bf16(ctx, static_cast<const uint16_t*>(drad), nprobes, dirs, K,
                                static_cast<float*>(ob.dev), split))) {
    return st;
  }
  if ((st = copy_out(ctx, ob))) return st;
  return finish(ctx, ob.host);
}

vlb_status vlb_sh_eval_envmap(vlb_ctx* ctx, const float* coeffs, uint32_t lmax, uint32_t w, uint32_t h, float scale,
                              float* out) {
  if (!ctx) return VLB_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (lmax != 2 && lmax != 3) return fail(ctx, VLB_ERR_INVALID, "lmax must be 2 or 3 (got %u)", lmax);
  if (!coeffs || !out || !w || !h || uint64_t(w) * h >= (1ull << 31)) return fail(ctx, VLB_ERR_INVALID, "bad image");
  const uint32_t K = k_of(lmax);
  vlb_status st;
  const void* dc;
  if ((st = stage_in(ctx, coeffs, size_t(K) * 12, "eval_coeffs", &dc))) return st;
  std::vector<float> col, row;
  pano_tables(w, h, false, col, row);
  void *dcol, *drow;
  if ((st = scratch(ctx, "eval_col", col.size() * 4, &dcol)) || (st = scratch(ctx, "eval_row", row.size() * 4, &drow)))
    return st;
  VLB_CUDA(ctx, cudaMemcpyAsync(dcol, col.data(), col.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  VLB_CUDA(ctx, cudaMemcpyAsync(drow, row.data(), row.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  OutBuf ob;
  if ((st = stage_out(ctx, out, size_t(w) * h * 12, "eval_out", &ob))) return st;
  {
    KScope k(ctx, "sh_eval_envmap");
    vlbk::launch_sh_eval_envmap(static_cast<const float*>(dc), K, w, h, scale, static_cast<const float2*>(dcol),
                                static_cast<const float4*>(drow), static_cast<float*>(ob.dev), ctx->stream);
  }
  if ((st = copy_out(ctx, ob))) return st;
  VLB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the host tables above must outlive their copies
  return finish(ctx, ob.host);
}

// ---- synthetic inputs ------------------------------------------------------------------------
vlb_status vlb_synth_box_scene(uint64_t seed, uint32_t nboxes, float* positions, uint32_t* indices, float* albedo,
                               uint32_t* nverts, uint32_t* ntris) {
  if (nboxes > (1u << 24)) return VLB_ERR_INVALID;
  const uint32_t nv = 8 + 8 * nboxes, nt = 10 + 12 * nboxes;
  if (nverts) *nverts = nv;
  if (ntris) *ntris = nt;
  if (!positions && !indices && !albedo) return VLB_OK;
  if (!positions || !indices || !albedo) return VLB_ERR_INVALID;
  // corner c = x + 2y + 4z of a box
  static const uint32_t room_quads[5][4] = {{0, 4, 5, 1}, {0, 2, 6, 4}, {1, 5, 7, 3}, {0, 1, 3, 2}, {4, 6, 7, 5}};
  static const uint32_t box_quads[6][4] = {{0, 4, 5, 1}, {2, 3, 7, 6}, {0, 2, 6, 4},
                                           {1, 5, 7, 3}, {0, 1, 3, 2}, {4, 6, 7, 5}};
  uint32_t tv = 0, tt = 0;
  auto corners = [&](const float* lo, const float* hi) {
    for (uint32_t c = 0; c < 8; ++c) {
      positions[3 * (tv + c)] = (c & 1) ? hi[0] : lo[0];
      positions[3 * (tv + c) + 1] = (c & 2) ? hi[1] : lo[1];
      positions[3 * (tv + c) + 2] = (c & 4) ? hi[2] : lo[2];
    }
  };
  auto quad = [&](const uint32_t* q, const float* rgb) {
    const uint32_t t[2][3] = {{q[0], q[1], q[2]}, {q[0], q[2], q[3]}};
    for (int i = 0; i < 2; ++i) {
      for (int k = 0; k < 3; ++k) { indices[3 * tt + k] = tv + t[i][k]; albedo[3 * tt + k] = rgb[k]; }
      ++tt;
    }
  };
  const float lo0[3] = {0.f, 0.f, 0.f}, hi0[3] = {1.f, 1.f, 1.f}, grey[3] = {0.5f, 0.5f, 0.5f};
  corners(lo0, hi0);
  for (auto& q : room_quads) quad(q, grey);
  tv += 8;
  SplitMix64 rng(seed ^ 0x5CE9E5CE9E5CE9EULL);
  for (uint32_t b = 0; b < nboxes; ++b) {
    float c[3], e[3], rgb[3];
    for (int a = 0; a < 3; ++a) c[a] = rng.range(0.1f, 0.9f);
    for (int a = 0; a < 3; ++a) e[a] = rng.range(0.05f, 0.2f);
    for (int a = 0; a < 3; ++a) rgb[a] = rng.range(0.2f, 0.8f);
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      volatile float half = e[a] * 0.5f;
      lo[a] = c[a] - half;
      hi[a] = c[a] + half;
    }
    corners(lo, hi);
    for (auto& q : box_quads) quad(q, rgb);
    tv += 8;
  }
  return VLB_OK;
}

vlb_status vlb_synth_cubemap(uint64_t seed, uint32_t n, float* out) {
  if (!out || n == 0 || n > 16384) return VLB_ERR_INVALID;
  SplitMix64 rng(seed ^ 0xC0BE0C0BE0C0BEULL);
  double mu[3][3], sharp[3], inten[3][3];
  for (int j = 0; j < 3; ++j) {
    rng.unit_dir(mu[j], false);
    sharp[j] = 20.0 + 180.0 * rng.uniform();
    for (int c = 0; c < 3; ++c) inten[j][c] = 1.0 + 49.0 * rng.uniform();
  }
  for (int f = 0; f < 6; ++f)
    for (uint32_t y = 0; y < n; ++y)
      for (uint32_t x = 0; x < n; ++x) {
        double d[3];
        cube_face_dir(f, 2.0 * (x + 0.5) / n - 1.0, 2.0 * (y + 0.5) / n - 1.0, d);
        double v[3] = {0.3, 0.3, 0.3};
        for (int j = 0; j < 3; ++j) {
          const double g = std::exp(sharp[j] * (d[0] * mu[j][0] + d[1] * mu[j][1] + d[2] * mu[j][2] - 1.0));
          for (int c = 0; c < 3; ++c) v[c] += inten[j][c] * g;
        }
        float* o = out + ((size_t(f) * n + y) * n + x) * 3;
        o[0] = float(v[0]); o[1] = float(v[1]); o[2] = float(v[2]);
      }
  return VLB_OK;
}

vlb_status vlb_synth_sun(uint64_t seed, float out_dir[3]) {
  if (!out_dir) return VLB_ERR_INVALID;
  SplitMix64 rng(seed ^ 0x5E45E45E45E45EULL);
  double d[3];
  rng.unit_dir(d, true);
  for (int a = 0; a < 3; ++a) out_dir[a] = float(d[a]);
  return VLB_OK;
}

}  // extern "C"
