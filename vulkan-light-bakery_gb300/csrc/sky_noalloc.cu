// sky_noalloc.cu -- skybox SH projection that allocates no memory.
//
// Some callers cannot allocate device memory at the moment they need a sky
// projection: a renderer that hands every byte of a fixed device-memory pool
// to its own sub-allocator, code running while another component holds the
// allocator, or a host that forbids cudaMalloc/cudaFree outside start-up.
// vlb_skybox_sh_noalloc serves them.  It runs the same kernels as
// vlb_skybox_sh (k_skybox.cu) and needs no context; its scratch -- slab
// partials, the cube-face solid-angle or panorama tables and the device error
// counters -- is one file-scope __device__ array of kNoAllocScratchBytes
// (557,312 bytes) that every GPU loading this library holds until the
// process exits.  Limits: one map per call, lmax 2 or 3, cubemap faces up to
// 256 x 256, panoramas up to 8192 x 8192; texels and out must be device
// memory of the current device.  Every call reuses the array and leaves its
// contents behind; the counters that must start at zero are cleared at the
// start of each call, so calls whose work overlaps on the GPU (several host
// threads, or several streams) race on the array and must be serialised by
// the caller.  The array's device address is looked up once per device and
// kept: after cudaDeviceReset (or a release of the device's primary context)
// the library's module is loaded again and the array may move, so calls
// after a reset are not supported.  Each call waits for its own work on the
// caller's stream (it reads the error counters back with an asynchronous
// copy on that stream, then synchronises the stream) before it returns.
#include <algorithm>
#include <mutex>

#include "vlb_device.cuh"
#include "vlb_internal.h"

namespace {

constexpr uint32_t kMaxSlabs = 512;
constexpr uint32_t kMaxValues = 48;  // 16 coefficients x RGB
constexpr uint32_t kMaxCubeFace = 256;
constexpr uint32_t kMaxPano = 8192;
constexpr size_t kPartialBytes = size_t(kMaxSlabs) * kMaxValues * 4;     // 98,304
constexpr size_t kTableBytes = size_t(kMaxCubeFace) * kMaxCubeFace * 4;  // 262,144
constexpr size_t kColBytes = size_t(kMaxPano) * 8;                       // 65,536
constexpr size_t kRowBytes = size_t(kMaxPano) * 16;                      // 131,072
constexpr size_t kErrBytes = 256;
constexpr size_t kNoAllocScratchBytes = kPartialBytes + kTableBytes + kColBytes + kRowBytes + kErrBytes;
static_assert(kNoAllocScratchBytes == 557312, "documented size");

// The scratch.  In host code this name is only a stand-in for the device
// array: host code never dereferences it or passes it to a kernel; it passes
// the device address obtained from cudaGetSymbolAddress instead.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Once per device, with that device current: the device address of the
// scratch array.  The first call on a device does this, so that first call
// should be made before any stream capture begins.
cudaError_t scratch_address(int dev, unsigned char** out) {
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_addr[dev]);
  return cudaSuccess;
}

// Panorama direction tables on the device (no host buffers): per column
// (cos phi, sin phi), per row (sin theta, cos theta, pixel weight) with the
// reference's PI (shaders/sh_common.h:1, :14-22; sh.comp:32-33).
__global__ void k_pano_tables(float2* col, float4* row, uint32_t w, uint32_t h, int shift) {
  const double pi = 3.1415926538;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < w) {
    double phi = 2.0 * pi * (double(i) + 0.5) / double(w);
    if (shift) phi -= pi / 2.0;
    col[i] = make_float2(float(cos(phi)), float(sin(phi)));
  }
  if (i < h) {
    const double th = pi * (double(i) + 0.5) / double(h);
    const double area = (2.0 * pi / w) * (pi / h);
    row[i] = make_float4(float(sin(th)), float(cos(th)), float(area * sin(th)), 0.f);
  }
}

bool on_device(const void* p, int dev) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == dev;
}

}  // namespace

extern "C" vlb_status vlb_skybox_sh_noalloc(const void* texels, vlb_texel_format fmt, vlb_sky_layout layout,
                                            uint32_t w, uint32_t h, uint32_t lmax, uint32_t flags, float* out,
                                            void* stream) {
  if (!texels || !out) return VLB_ERR_INVALID;
  if (lmax != 2 && lmax != 3) return VLB_ERR_INVALID;
  if (flags & ~uint32_t(VLB_SKY_REF_BGRA_SWAP)) return VLB_ERR_INVALID;
  if (fmt != VLB_TEXEL_RGB32F && fmt != VLB_TEXEL_RGBA8) return VLB_ERR_INVALID;
  if (layout != VLB_SKY_CUBEMAP && layout != VLB_SKY_PANORAMA && layout != VLB_SKY_ENVMAP) return VLB_ERR_INVALID;
  if (!w || !h) return VLB_ERR_INVALID;
  if (layout == VLB_SKY_CUBEMAP && (w != h || w > kMaxCubeFace)) return VLB_ERR_INVALID;
  if (layout != VLB_SKY_CUBEMAP && (w > kMaxPano || h > kMaxPano)) return VLB_ERR_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return VLB_ERR_CUDA;
  if (!on_device(texels, dev) || !on_device(out, dev)) return VLB_ERR_INVALID;
  unsigned char* base = nullptr;
  if (scratch_address(dev, &base) != cudaSuccess) { cudaGetLastError(); return VLB_ERR_CUDA; }
  int num_sms = 0;
  if (cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return VLB_ERR_CUDA;
  float* partial = reinterpret_cast<float*>(base);
  float* table = reinterpret_cast<float*>(base + kPartialBytes);
  float2* col = reinterpret_cast<float2*>(base + kPartialBytes + kTableBytes);
  float4* row = reinterpret_cast<float4*>(base + kPartialBytes + kTableBytes + kColBytes);
  int* err = reinterpret_cast<int*>(base + kPartialBytes + kTableBytes + kColBytes + kRowBytes);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // A launch error the caller left pending on this thread is not this call's:
  // it is neither cleared nor reported here.
  const cudaError_t prior = cudaPeekAtLastError();
  auto launch_failed = [prior]() {
    if (prior != cudaSuccess) return false;
    if (cudaPeekAtLastError() == cudaSuccess) return false;
    cudaGetLastError();  // this call's own launch error: clear it
    return true;
  };

  const uint32_t T = layout == VLB_SKY_CUBEMAP ? 6 * w * w : w * h;
  const uint32_t TB = fmt == VLB_TEXEL_RGB32F ? 12 : 4;
  const uint32_t K = (lmax + 1) * (lmax + 1), V = 3 * K;
  vlbk::SkyboxArgs a{};
  a.texels = texels; a.fmt = fmt; a.layout = layout; a.w = w; a.h = h; a.count = 1; a.lmax = lmax;
  a.flags = flags; a.texels_per_map = T; a.err = err;
  // the work split of vlb_skybox_sh within kMaxSlabs partials (8 per slab):
  // maps above 64 x 8192 texels get wider slabs
  vlbk::skybox_plan(a, kMaxSlabs / vlbk::kSkyPartialsPerSlab);
  const uint32_t spm = a.slabs_per_map;
  if (spm * vlbk::kSkyPartialsPerSlab > kMaxSlabs) return VLB_ERR_INVALID;
  a.partial = partial;
  if (cudaMemsetAsync(err, 0, vlbk::kErrSlots * sizeof(int), s) != cudaSuccess) return VLB_ERR_CUDA;
  if (layout == VLB_SKY_CUBEMAP) {
    vlbk::launch_cube_solid_angle(table, w, s);
    a.solid_angle = table;
  } else {
    const uint32_t n = std::max(w, h);
    k_pano_tables<<<(n + 255) / 256, 256, 0, s>>>(col, row, w, h, layout == VLB_SKY_PANORAMA);
    a.col_tab = col; a.row_tab = row;
  }
  if (launch_failed()) return VLB_ERR_CUDA;
  const bool tma = (reinterpret_cast<uintptr_t>(texels) % 16 == 0) && ((uint64_t(T) * TB) % 16 == 0);
  const int per_map = vlbk::launch_skybox_sh(a, tma, num_sms, s);
  if (launch_failed()) return VLB_ERR_CUDA;
  vlbk::launch_sh_finalize(partial, 1, uint32_t(per_map), V, out, s);
  if (launch_failed()) return VLB_ERR_CUDA;
  // the error counters come back on the caller's stream (no legacy-stream copy)
  int herr[vlbk::kErrSlots];
  if (cudaMemcpyAsync(herr, err, sizeof herr, cudaMemcpyDeviceToHost, s) != cudaSuccess) return VLB_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return VLB_ERR_CUDA;
  if (herr[vlbk::kErrTimeout]) return VLB_ERR_TIMEOUT;
  for (int i = 0; i < vlbk::kErrSlots; ++i)
    if (herr[i]) return VLB_ERR_INTERNAL;
  return VLB_OK;
}
