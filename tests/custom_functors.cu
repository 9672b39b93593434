// Test support: two functor sets that are no preset of the library, compiled
// against include/nvpro_pyramid_cuda.hpp as a caller of the library would
// compile its own, and exported as custom pipeline pairs.
#include <cuda_runtime.h>

#include "nvpro_pyramid_cuda.hpp"

// A depth pyramid (hierarchical Z): one FP32 channel, the maximum of each
// footprint.  REDUCE ignores the weights; REDUCE2 / REDUCE4 are the reference's
// defaults built from it.
struct MaxDepth : nvpro_pyramid::StatelessFunctors {
  using Texel = float;
  using Value = float;
  __device__ float load(float t) const { return t; }
  __device__ float store(float v) const { return v; }
  __device__ float reduce(float, float v0, float, float v1, float, float v2) const {
    return fmaxf(fmaxf(v0, v1), v2);
  }
};

// RGBA 16-bit unorm texels with linear FP32 arithmetic: LOAD c / 65535, STORE
// uint(clamp(v, 0, 1) * 65535 + 0.5), REDUCE a0 v0 + a1 v1 + a2 v2 left to
// right with every operation rounded; REDUCE2 / REDUCE4 from the defaults.
struct Rgba16Unorm : nvpro_pyramid::StatelessFunctors {
  using Texel = ushort4;
  using Value = float4;
  __device__ static float unorm(unsigned short c) { return __fdiv_rn(float(c), 65535.0f); }
  __device__ static unsigned short pack(float v) {
    const float x = fminf(fmaxf(v, 0.0f), 1.0f);
    return static_cast<unsigned short>(__float2uint_rz(__fadd_rn(__fmul_rn(x, 65535.0f), 0.5f)));
  }
  __device__ static float mac(float a0, float v0, float a1, float v1, float a2, float v2) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a0, v0), __fmul_rn(a1, v1)), __fmul_rn(a2, v2));
  }
  __device__ float4 load(const ushort4& t) const { return make_float4(unorm(t.x), unorm(t.y), unorm(t.z), unorm(t.w)); }
  __device__ ushort4 store(const float4& v) const { return make_ushort4(pack(v.x), pack(v.y), pack(v.z), pack(v.w)); }
  __device__ float4 reduce(float a0, const float4& v0, float a1, const float4& v1, float a2, const float4& v2) const {
    return make_float4(mac(a0, v0.x, a1, v1.x, a2, v2.x), mac(a0, v0.y, a1, v1.y, a2, v2.y),
                       mac(a0, v0.z, a1, v1.z, a2, v2.z), mac(a0, v0.w, a1, v1.w, a2, v2.w));
  }
};

// which 0: MaxDepth, 1: Rgba16Unorm.  fast may be NULL (general pipeline only).
extern "C" __attribute__((visibility("default"))) NvproPyramidResult customCreatePipelines(
    int which, NvproPyramidPipeline* general, NvproPyramidPipeline* fast) {
  if (which == 0) return nvpro_pyramid::createPipelines<MaxDepth>(general, fast);
  if (which == 1) return nvpro_pyramid::createPipelines<Rgba16Unorm>(general, fast);
  return NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT;
}
