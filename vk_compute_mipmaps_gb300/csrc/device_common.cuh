// device_common.cuh -- device-side building blocks shared by every kernel:
// the reference's customisation points (NVPRO_PYRAMID_LOAD / REDUCE / REDUCE2 /
// REDUCE4 / STORE, nvpro_pyramid.glsl:27-120) as device functors, and the
// exact sRGB codec.
//
// Arithmetic rule: every multiply and add is a separately rounded IEEE FP32
// operation in the order the reference macros write it (__fmul_rn/__fadd_rn
// forbid FMA contraction); 1/(2n+1) is correctly rounded (__frcp_rn).
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/nvpro_pyramid_cuda.hpp"
#include "internal.h"
#include "srgb_tables.h"

namespace nvpyr {

// ---------------------------------------------------------------------------
// Reduction operators of the sRGBA8 preset (srgba8_mipmap_preamble.glsl:24-38),
// shared by the float presets.

__device__ __forceinline__ float4 f4add(float4 a, float4 b) {
  return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}
__device__ __forceinline__ float4 f4scale(float s, float4 a) {
  return make_float4(__fmul_rn(s, a.x), __fmul_rn(s, a.y), __fmul_rn(s, a.z), __fmul_rn(s, a.w));
}

// NVPRO_PYRAMID_REDUCE4: 0.25 * ((v00 + v01) + (v10 + v11))
__device__ __forceinline__ float4 reduce4(float4 v00, float4 v01, float4 v10, float4 v11) {
  return f4scale(0.25f, f4add(f4add(v00, v01), f4add(v10, v11)));
}
// NVPRO_PYRAMID_REDUCE2: 0.5 * (v0 + v1)
__device__ __forceinline__ float4 reduce2(float4 v0, float4 v1) { return f4scale(0.5f, f4add(v0, v1)); }
// NVPRO_PYRAMID_REDUCE: a0 * v0 + a1 * v1 + a2 * v2
__device__ __forceinline__ float4 reduce3(float a0, float4 v0, float a1, float4 v1, float a2, float4 v2) {
  return f4add(f4add(f4scale(a0, v0), f4scale(a1, v1)), f4scale(a2, v2));
}

// 3-tap weights of the general pipeline (nvpro_pyramid.glsl:582-586, :639-643).
using nvpro_pyramid::detail::Weights3;
using nvpro_pyramid::detail::weights3;

// REDUCE4 of a 2x2 block in the fast pipeline's order for its level
// (fastVerticalFirst): vertical pairs first, or horizontal pairs first.
__device__ __forceinline__ float4 fastReduce(bool vertical, float4 tl, float4 tr, float4 bl, float4 br) {
  return vertical ? reduce4(tl, bl, tr, br) : reduce4(tl, tr, bl, br);
}

// ---------------------------------------------------------------------------
// Exact sRGB codec.

static __constant__ uint32_t c_srgbDecodeBits[256] = {NVPYR_SRGB_DECODE_BITS};
static __constant__ uint32_t c_alphaDecodeBits[256] = {NVPYR_ALPHA_DECODE_BITS};
static __constant__ uint32_t c_srgbThresholdBits[256] = {NVPYR_SRGB_ENCODE_THRESHOLD_BITS};

// The three tables in shared memory, one copy (portable kernels).
struct SrgbTablesSmem {
  float decode[256];
  float alpha[256];
  float thr[256];
};

__device__ __forceinline__ void loadSrgbTables(SrgbTablesSmem* t) {
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) {
    t->decode[i] = __uint_as_float(c_srgbDecodeBits[i]);
    t->alpha[i] = __uint_as_float(c_alphaDecodeBits[i]);
    t->thr[i] = __uint_as_float(c_srgbThresholdBits[i]);
  }
}

// sRGB code of a linear value: the number of thresholds <= x.
__device__ __forceinline__ uint32_t srgbEncodeSearch(float x, const float* thr) {
  uint32_t n = 0;
#pragma unroll
  for (uint32_t step = 128; step > 0; step >>= 1)
    if (n + step <= 255 && thr[n + step - 1] <= x) n += step;
  return n;
}

// srgbFromLinearVec's alpha (srgba8_mipmap_preamble.glsl:125):
// clamp(uint(a * 255.0f + 0.5f), 0u, 255u); negative and NaN give 0.
__device__ __forceinline__ uint32_t alphaEncode(float a) {
  const float s = __fadd_rn(__fmul_rn(a, 255.0f), 0.5f);
  return min(__float2uint_rz(s), 255u);
}

// ---------------------------------------------------------------------------
// Texel I/O per preset (NVPRO_PYRAMID_LOAD / NVPRO_PYRAMID_STORE).

template <uint32_t P>
struct TexelIO;

template <>
struct TexelIO<kSrgba8> {
  static constexpr uint32_t kBytes = 4;
  const SrgbTablesSmem* t;
  __device__ __forceinline__ float4 decode(uint32_t w) const {
    return make_float4(t->decode[w & 255u], t->decode[(w >> 8) & 255u], t->decode[(w >> 16) & 255u],
                       t->alpha[w >> 24]);
  }
  __device__ __forceinline__ uint32_t encode(float4 v) const {
    return srgbEncodeSearch(v.x, t->thr) | srgbEncodeSearch(v.y, t->thr) << 8 |
           srgbEncodeSearch(v.z, t->thr) << 16 | alphaEncode(v.w) << 24;
  }
  __device__ __forceinline__ float4 load(const uint8_t* p) const { return decode(*(const uint32_t*)p); }
  __device__ __forceinline__ void store(uint8_t* p, float4 v) const { *(uint32_t*)p = encode(v); }
};

template <>
struct TexelIO<kRgba32f> {
  static constexpr uint32_t kBytes = 16;
  const void* t;
  __device__ __forceinline__ float4 load(const uint8_t* p) const { return *(const float4*)p; }
  __device__ __forceinline__ void store(uint8_t* p, float4 v) const { *(float4*)p = v; }
};

template <>
struct TexelIO<kRgba16f> {
  static constexpr uint32_t kBytes = 8;
  const void* t;
  __device__ __forceinline__ float4 load(const uint8_t* p) const {
    const uint2 u = *(const uint2*)p;
    const __half2 a = *reinterpret_cast<const __half2*>(&u.x);
    const __half2 b = *reinterpret_cast<const __half2*>(&u.y);
    return make_float4(__low2float(a), __high2float(a), __low2float(b), __high2float(b));
  }
  __device__ __forceinline__ void store(uint8_t* p, float4 v) const {
    const __half2 a = __floats2half2_rn(v.x, v.y);
    const __half2 b = __floats2half2_rn(v.z, v.w);
    uint2 u;
    u.x = *reinterpret_cast<const uint32_t*>(&a);
    u.y = *reinterpret_cast<const uint32_t*>(&b);
    *(uint2*)p = u;
  }
};

// F16_SHARED (srgba8_mipmap_preamble.glsl:103-108): f16vec4(v) and back;
// each channel rounded to binary16, nearest even.
__device__ __forceinline__ float4 f16RoundTrip(float4 v) {
  return make_float4(__half2float(__float2half_rn(v.x)), __half2float(__float2half_rn(v.y)),
                     __half2float(__float2half_rn(v.z)), __half2float(__float2half_rn(v.w)));
}

__device__ __forceinline__ uint8_t* texelAddr(const LevelView& v, uint32_t x, uint32_t y, uint32_t bytes) {
  return v.ptr + (uint64_t)y * v.pitch + (uint64_t)x * bytes;
}

}  // namespace nvpyr
