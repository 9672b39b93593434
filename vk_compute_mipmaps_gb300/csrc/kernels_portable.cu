// kernels_portable.cu -- the fast and general pyramid pipelines for any
// preset and any level layout (per-level pointers and row pitches), with plain
// global loads and stores: the library's built-in presets as functor sets of
// nvpro_pyramid_cuda.hpp, whose fastKernel / general1Kernel / general2Kernel
// templates every custom pipeline instantiates too.  These kernels define the
// library's semantics; the TMA, column-strip and small-dispatch kernels are
// faster equivalents for the sRGBA8 preset and produce identical bytes.
//
// Semantics follow nvpro_pyramid.glsl dispatch by dispatch: a fast dispatch of
// n levels reduces each 2^n x 2^n tile of level L with 2x2 box filters whose
// operand order is fastVerticalFirst(n, k); a general dispatch of 1 or 2 levels
// applies the 1..3-tap energy-conserving kernel.  Values stay FP32 inside a
// dispatch and are quantised only by the STORE of each level, except the
// hand-off level of a pipeline with a shared-memory format.
#include <algorithm>

#include "../../include/nvpro_pyramid_cuda.hpp"
#include "device_common.cuh"

namespace nvpyr {
namespace {

constexpr uint32_t kThreads = 256;

// The sRGBA8 preset (srgba8_mipmap_preamble.glsl:10-128): texelFetch of an
// sRGB texture (the exact decode tables), REDUCE / REDUCE2 / REDUCE4 in FP32
// with every operation rounded separately, srgbFromLinearVec on store.
struct Srgba8Functors {
  using Texel = uint32_t;
  using Value = float4;
  struct Tables {
    SrgbTablesSmem t;
  };
  __device__ static void initTables(Tables& tb, unsigned, unsigned) { loadSrgbTables(&tb.t); }
  const SrgbTablesSmem* t;
  __device__ explicit Srgba8Functors(const Tables& tb) : t(&tb.t) {}
  __device__ float4 load(uint32_t w) const { return TexelIO<kSrgba8>{t}.decode(w); }
  __device__ uint32_t store(const float4& v) const { return TexelIO<kSrgba8>{t}.encode(v); }
  __device__ float4 reduce(float a0, const float4& v0, float a1, const float4& v1, float a2, const float4& v2) const {
    return reduce3(a0, v0, a1, v1, a2, v2);
  }
  __device__ float4 reduce2(const float4& v0, const float4& v1) const { return nvpyr::reduce2(v0, v1); }
  __device__ float4 reduce4(const float4& v00, const float4& v01, const float4& v10, const float4& v11) const {
    return nvpyr::reduce4(v00, v01, v10, v11);
  }
};

// SRGB_SHARED (srgba8_mipmap_preamble.glsl:60-101): the hand-off values as
// the texel's sRGBA8 code, decoded again with the load tables.
struct Srgba8SrgbShared : Srgba8Functors {
  using Srgba8Functors::Srgba8Functors;
  using SharedValue = uint32_t;
  __device__ uint32_t toShared(const float4& v) const { return store(v); }
  __device__ float4 fromShared(uint32_t s) const { return load(s); }
};

// F16_SHARED (srgba8_mipmap_preamble.glsl:103-108): each channel as binary16.
struct Srgba8F16Shared : Srgba8Functors {
  using Srgba8Functors::Srgba8Functors;
  using SharedValue = float4;  // the binary16 values, widened exactly
  __device__ float4 toShared(const float4& v) const { return f16RoundTrip(v); }
  __device__ float4 fromShared(const float4& s) const { return s; }
};

// Linear RGBA FP32 texels.
struct Rgba32fFunctors : nvpro_pyramid::StatelessFunctors {
  using Texel = float4;
  using Value = float4;
  __device__ float4 load(const float4& t) const { return t; }
  __device__ float4 store(const float4& v) const { return v; }
  __device__ float4 reduce(float a0, const float4& v0, float a1, const float4& v1, float a2, const float4& v2) const {
    return reduce3(a0, v0, a1, v1, a2, v2);
  }
  __device__ float4 reduce2(const float4& v0, const float4& v1) const { return nvpyr::reduce2(v0, v1); }
  __device__ float4 reduce4(const float4& v00, const float4& v01, const float4& v10, const float4& v11) const {
    return nvpyr::reduce4(v00, v01, v10, v11);
  }
};

// Linear RGBA with FP16 storage and FP32 arithmetic (round to nearest even).
struct Rgba16fFunctors : Rgba32fFunctors {
  using Texel = uint2;
  __device__ float4 load(const uint2& u) const { return TexelIO<kRgba16f>{nullptr}.load(reinterpret_cast<const uint8_t*>(&u)); }
  __device__ uint2 store(const float4& v) const {
    uint2 u;
    TexelIO<kRgba16f>{nullptr}.store(reinterpret_cast<uint8_t*>(&u), v);
    return u;
  }
};

// The dispatch as the header's kernels take it.
nvpro_pyramid::detail::DispatchArg toArg(const DispatchParams& p) {
  nvpro_pyramid::detail::DispatchArg a{};
  a.isFast = p.isFast;
  a.n = p.levelCount;
  a.groups = p.groups;
  for (uint32_t k = 0; k <= p.levelCount; ++k)
    a.lv[k] = nvpro_pyramid::detail::LevelArg{p.lv[k].ptr, p.lv[k].pitch, p.lv[k].w, p.lv[k].h, p.imageStride[k]};
  return a;
}

template <class F>
cudaError_t launchWith(const DispatchParams& p, cudaStream_t stream, uint32_t* launches) {
  return nvpro_pyramid::detail::launchDispatch<F>(toArg(p), p.batch, stream, launches);
}

// Level L+k of this CTA's image (blockIdx.z of a strided batch).
__device__ __forceinline__ LevelView levelOf(const DispatchParams& p, uint32_t k) {
  LevelView v = p.lv[k];
  v.ptr += uint64_t(blockIdx.z) * p.imageStride[k];
  return v;
}

// ---------------------------------------------------------------------------
// Linear blit of one level (vkCmdBlitImage with VK_FILTER_LINEAR, the
// fallback of the demo's "generalblit" mode, demo_app/mipmap_pipelines.cpp:
// 408-423): destination texel (x, y) samples the source at
// ((x + 0.5) srcW / dstW, (y + 0.5) srcH / dstH), bilinear on decoded values
// with clamp-to-edge, each FP32 operation rounded as the header states.
struct BlitAxis {
  uint32_t i0, i1;  // source texels (clamped)
  float a;          // weight of i1
};

__device__ __forceinline__ BlitAxis blitAxis(uint32_t x, uint32_t srcSize, uint32_t dstSize) {
  const float scale = __fdiv_rn(__uint2float_rn(srcSize), __uint2float_rn(dstSize));
  const float u = __fsub_rn(__fmul_rn(__fadd_rn(__uint2float_rn(x), 0.5f), scale), 0.5f);
  const float f = floorf(u);
  BlitAxis r;
  r.a = __fsub_rn(u, f);
  const int i = int(f);
  r.i0 = uint32_t(min(max(i, 0), int(srcSize) - 1));
  r.i1 = uint32_t(min(max(i + 1, 0), int(srcSize) - 1));
  return r;
}

__device__ __forceinline__ float4 lerp4(float4 t0, float4 t1, float a) {
  const float b = __fsub_rn(1.0f, a);
  return f4add(f4scale(b, t0), f4scale(a, t1));
}

template <uint32_t P>
__global__ void __launch_bounds__(kThreads) portableBlitKernel(DispatchParams p) {
  __shared__ SrgbTablesSmem tabs;
  if (P == kSrgba8) {
    loadSrgbTables(&tabs);
    __syncthreads();
  }
  TexelIO<P> io;
  io.t = &tabs;
  constexpr uint32_t B = TexelIO<P>::kBytes;
  const LevelView src = levelOf(p, 0), dst = levelOf(p, 1);
  const uint64_t total = uint64_t(dst.w) * dst.h;
  for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < total; i += uint64_t(gridDim.x) * kThreads) {
    const uint32_t x = uint32_t(i % dst.w), y = uint32_t(i / dst.w);
    const BlitAxis ax = blitAxis(x, src.w, dst.w), ay = blitAxis(y, src.h, dst.h);
    const float4 r0 = lerp4(io.load(texelAddr(src, ax.i0, ay.i0, B)), io.load(texelAddr(src, ax.i1, ay.i0, B)), ax.a);
    const float4 r1 = lerp4(io.load(texelAddr(src, ax.i0, ay.i1, B)), io.load(texelAddr(src, ax.i1, ay.i1, B)), ax.a);
    io.store(texelAddr(dst, x, y, B), lerp4(r0, r1, ay.a));
  }
}

template <uint32_t P>
cudaError_t launchBlit(const DispatchParams& p, cudaStream_t stream, uint32_t* launches) {
  const uint64_t total = uint64_t(p.lv[1].w) * p.lv[1].h;
  const uint64_t blocks = std::min<uint64_t>((total + kThreads - 1) / kThreads, 152u * 64u);
  portableBlitKernel<P><<<dim3(uint32_t(blocks), 1, p.batch), kThreads, 0, stream>>>(p);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace

cudaError_t launchPortable(const DispatchParams& p, cudaStream_t stream, uint32_t* launches) {
  switch (p.preset) {
    case kSrgba8:
      if (p.isBlit) return launchBlit<kSrgba8>(p, stream, launches);
      if (p.sharedFmt == kSharedSrgb) return launchWith<Srgba8SrgbShared>(p, stream, launches);
      if (p.sharedFmt == kSharedF16) return launchWith<Srgba8F16Shared>(p, stream, launches);
      return launchWith<Srgba8Functors>(p, stream, launches);
    case kRgba32f:
      return p.isBlit ? launchBlit<kRgba32f>(p, stream, launches) : launchWith<Rgba32fFunctors>(p, stream, launches);
    case kRgba16f:
      return p.isBlit ? launchBlit<kRgba16f>(p, stream, launches) : launchWith<Rgba16fFunctors>(p, stream, launches);
  }
  return cudaErrorInvalidValue;
}

}  // namespace nvpyr
