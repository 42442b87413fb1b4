// k_image.cu -- RGBA8 encoding of radiance images (debug env maps).
//
// The reference stores every env-map texel into an R8G8B8A8 UNORM image
// (src/baker/env_map_generator.hpp:39): env_map.rchit:101 and main.rmiss:40
// pass the radiance through sRGB() (main.rchit:49-56: 12.92 x below
// 0.0031308, else 1.055 x^(1/2.4) - 0.055) and env_map.rgen:27 writes it with
// alpha 1; sh_sum.comp:51 writes 1250 x the reconstruction without sRGB.
// UNORM conversion clamps to [0, 1] and rounds v * 255 to the nearest integer.
#include <algorithm>

#include "vlb_internal.h"

namespace vlbk {

__device__ __forceinline__ float srgb_oetf(float v) {
  return v < 0.0031308f ? v * 12.92f : 1.055f * powf(v, 1.0f / 2.4f) - 0.055f;
}

__global__ void k_encode_rgba8(const float* __restrict__ rgb, size_t n, float scale, uint32_t srgb,
                               uchar4* __restrict__ out) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    float c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float v = scale * rgb[3 * i + k];
      if (srgb) v = srgb_oetf(v);
      v = fminf(fmaxf(v, 0.f), 1.f);  // NaN -> 0
      c[k] = v;
    }
    out[i] = make_uchar4(uint8_t(__float2uint_rn(c[0] * 255.f)), uint8_t(__float2uint_rn(c[1] * 255.f)),
                         uint8_t(__float2uint_rn(c[2] * 255.f)), 255);
  }
}

void launch_encode_rgba8(const float* rgb, size_t n, float scale, uint32_t srgb, uint8_t* out, int num_sms,
                         cudaStream_t s) {
  if (!n) return;
  const size_t blocks = std::min<size_t>((n + 255) / 256, size_t(num_sms) * 8);
  k_encode_rgba8<<<uint32_t(blocks), 256, 0, s>>>(rgb, n, scale, srgb, reinterpret_cast<uchar4*>(out));
}

}  // namespace vlbk
