/*
 * nvpro_pyramid_cuda.hpp -- the customisation points of nvpro_pyramid as
 * device-functor template parameters (CUDA C++; compile with nvcc).
 *
 * The reference is a GLSL template: a shader defines NVPRO_PYRAMID_TYPE,
 * NVPRO_PYRAMID_LOAD, NVPRO_PYRAMID_REDUCE (and optionally REDUCE2, REDUCE4,
 * SHARED_TYPE / SHARED_LOAD / SHARED_STORE), includes nvpro_pyramid.glsl and
 * gets the fast and the general pipeline (nvpro_pyramid/nvpro_pyramid.glsl:
 * 27-120, defaults :148-207).  Here a C++ type F plays the macros' part, and
 * nvpro_pyramid::createPipelines<F>() gives the fast and general pipelines of
 * F as two NvproPyramidPipeline handles of the C ABI: nvproCmdPyramidDispatch
 * and nvproPyramidGenerate then run F's kernels with the reference's schedule,
 * quantisation points and operation order, exactly as for the built-in
 * presets (which are instances of the same templates: the library's portable
 * kernels are fastKernel / general1Kernel / general2Kernel of its sRGBA8,
 * RGBA32F and RGBA16F functor sets).
 *
 * The functor set F (a trivially copyable class type):
 *
 *   using Texel = ...;  // what one texel of a level holds in memory
 *                       // (NVPRO_PYRAMID_LOAD / STORE address memory in the
 *                       // reference; here the library addresses levels and
 *                       // F converts texels)
 *   using Value = ...;  // NVPRO_PYRAMID_TYPE: trivially constructible, at
 *                       // most 32 bytes (the reference's recommendation)
 *   struct Tables {...};  // state in shared memory per CTA (may be empty),
 *   __device__ static void initTables(Tables& t, unsigned thread, unsigned threads);
 *                       // fills it cooperatively; a __syncthreads follows
 *   __device__ F(const Tables& t);  // (or default-constructible) a handle per thread
 *
 *   __device__ Value load(const Texel& t) const;   // NVPRO_PYRAMID_LOAD
 *   __device__ Texel store(const Value& v) const;  // NVPRO_PYRAMID_STORE
 *   __device__ Value reduce(float a0, const Value& v0, float a1, const Value& v1,
 *                           float a2, const Value& v2) const;  // NVPRO_PYRAMID_REDUCE
 * optional:
 *   __device__ Value reduce2(const Value& v0, const Value& v1) const;
 *       // NVPRO_PYRAMID_REDUCE2; default reduce(0.5, v0, 0.5, v1, 0, v1)
 *   __device__ Value reduce4(const Value& v00, const Value& v01, const Value& v10,
 *                            const Value& v11) const;
 *       // NVPRO_PYRAMID_REDUCE4; default reduce2(reduce2(v00, v01), reduce2(v10, v11))
 *   using SharedValue = ...;  // NVPRO_PYRAMID_SHARED_TYPE, with
 *   __device__ SharedValue toShared(const Value& v) const;    // SHARED_STORE
 *   __device__ Value fromShared(const SharedValue& s) const;  // SHARED_LOAD
 *       // applied to the values a dispatch hands on from its hand-off level
 *       // (nvpro_pyramid::sharedHandoffLevel); default: none.
 * nvpro_pyramid::StatelessFunctors provides an empty Tables and initTables.
 *
 * Operand order: LOAD_REDUCE4 loads (x, y), (x, y+1), (x+1, y), (x+1, y+1) and
 * calls reduce4 with them in that order (nvpro_pyramid.glsl:180-188); the
 * deeper fast levels call reduce4 with the order fastVerticalFirst(n, k)
 * gives; general levels reduce each column vertically first, then the row
 * (reduceStoreSample_, :575-656), with reduce for three taps and reduce2 for
 * two.  For a bit-exact result the functors' arithmetic must not be contracted
 * across calls; the library's own sets use separately rounded intrinsics.
 */
#ifndef NVPRO_PYRAMID_CUDA_HPP_
#define NVPRO_PYRAMID_CUDA_HPP_

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>
#include <utility>

#include "nvpro_pyramid_cuda.h"
#include "nvpro_pyramid_rules.h"

namespace nvpro_pyramid {

/* Base for functor sets that need no shared-memory state. */
struct StatelessFunctors {
  struct Tables {};
  __device__ static void initTables(Tables&, unsigned, unsigned) {}
};

namespace detail {

// ---------------------------------------------------------------------------
// The reference's defaults for the optional customisation points.

template <class F, class = void>
struct HasReduce2 : std::false_type {};
template <class F>
struct HasReduce2<F, std::void_t<decltype(std::declval<const F&>().reduce2(std::declval<typename F::Value>(),
                                                                           std::declval<typename F::Value>()))>>
    : std::true_type {};

template <class F, class = void>
struct HasReduce4 : std::false_type {};
template <class F>
struct HasReduce4<F, std::void_t<decltype(std::declval<const F&>().reduce4(
                         std::declval<typename F::Value>(), std::declval<typename F::Value>(),
                         std::declval<typename F::Value>(), std::declval<typename F::Value>()))>> : std::true_type {};

template <class F, class = void>
struct HasShared : std::false_type {};
template <class F>
struct HasShared<F, std::void_t<typename F::SharedValue>> : std::true_type {};

template <class F>
__device__ __forceinline__ typename F::Value reduce2(const F& f, const typename F::Value& v0,
                                                     const typename F::Value& v1) {
  if constexpr (HasReduce2<F>::value)
    return f.reduce2(v0, v1);
  else
    return f.reduce(0.5f, v0, 0.5f, v1, 0.0f, v1);  // nvpro_pyramid.glsl:164-167
}

template <class F>
__device__ __forceinline__ typename F::Value reduce4(const F& f, const typename F::Value& v00,
                                                     const typename F::Value& v01, const typename F::Value& v10,
                                                     const typename F::Value& v11) {
  if constexpr (HasReduce4<F>::value) {
    return f.reduce4(v00, v01, v10, v11);
  } else {  // nvpro_pyramid.glsl:169-177
    const typename F::Value a = reduce2(f, v00, v01), b = reduce2(f, v10, v11);
    return reduce2(f, a, b);
  }
}

// REDUCE4 of a 2x2 block in the fast pipeline's order for its level.
template <class F>
__device__ __forceinline__ typename F::Value fastReduce(const F& f, bool vertical, const typename F::Value& tl,
                                                        const typename F::Value& tr, const typename F::Value& bl,
                                                        const typename F::Value& br) {
  return vertical ? reduce4(f, tl, bl, tr, br) : reduce4(f, tl, tr, bl, br);
}

// The value handed on from the hand-off level: SHARED_LOAD(SHARED_STORE(v)).
template <class F>
__device__ __forceinline__ typename F::Value handOff(const F& f, const typename F::Value& v) {
  if constexpr (HasShared<F>::value)
    return f.fromShared(f.toShared(v));
  else
    return v;
}

template <class F>
__device__ __forceinline__ F makeFunctors(const typename F::Tables& t) {
  if constexpr (std::is_constructible<F, const typename F::Tables&>::value)
    return F(t);
  else
    return F();
}

// 3-tap weights of the general pipeline (nvpro_pyramid.glsl:582-586,
// :639-643) for destination size n and coordinate i: w0 = (n - i) / (2n + 1),
// w1 = n / (2n + 1), w2 = 1 - w0 - w1, with 1 / (2n + 1) correctly rounded and
// every operation rounded separately.
struct Weights3 {
  float w0, w1, w2;
};
__device__ __forceinline__ Weights3 weights3(uint32_t n, uint32_t i) {
  const float nf = __uint2float_rn(n);
  const float rcp = __frcp_rn(__fadd_rn(__fmul_rn(2.0f, nf), 1.0f));
  Weights3 w;
  w.w0 = __fmul_rn(rcp, __fsub_rn(nf, __uint2float_rn(i)));
  w.w1 = __fmul_rn(rcp, nf);
  w.w2 = __fsub_rn(__fsub_rn(1.0f, w.w0), w.w1);
  return w;
}

// ---------------------------------------------------------------------------
// One dispatch as the kernels see it.

struct LevelArg {
  uint8_t* ptr;          // texel (0, 0) of image 0
  uint64_t pitch;        // bytes between rows
  uint32_t w, h;
  uint64_t imageStride;  // bytes between images (strided batches, grid z)
};

struct DispatchArg {
  uint32_t isFast;
  uint32_t n;       // levels filled
  uint64_t groups;  // reference workgroups dispatched (coverage)
  LevelArg lv[7];   // levels L .. L+n
};

template <class F>
__device__ __forceinline__ typename F::Value loadAt(const F& f, const LevelArg& v, uint32_t x, uint32_t y) {
  const uint8_t* p =
      v.ptr + uint64_t(blockIdx.z) * v.imageStride + uint64_t(y) * v.pitch + uint64_t(x) * sizeof(typename F::Texel);
  return f.load(*reinterpret_cast<const typename F::Texel*>(p));
}

template <class F>
__device__ __forceinline__ void storeAt(const F& f, const LevelArg& v, uint32_t x, uint32_t y,
                                        const typename F::Value& val) {
  uint8_t* p =
      v.ptr + uint64_t(blockIdx.z) * v.imageStride + uint64_t(y) * v.pitch + uint64_t(x) * sizeof(typename F::Texel);
  *reinterpret_cast<typename F::Texel*>(p) = f.store(val);
}

constexpr uint32_t kRegion = 64;  // fast kernel: a 64x64 region of level L per CTA
constexpr uint32_t kThreads = 256;
constexpr uint32_t kG2Tile = 16;  // two-level general kernel: a 16x16 tile of level L+2 per CTA
constexpr uint32_t kG2Win = 2 * kG2Tile + 1;

template <class F>
struct FunctorChecks {
  static_assert(sizeof(typename F::Value) <= 32, "NVPRO_PYRAMID_TYPE should be at most 32 bytes");
  static_assert(std::is_trivially_default_constructible<typename F::Value>::value,
                "Value must be trivially constructible (it lives in shared memory)");
  static_assert(std::is_trivially_default_constructible<typename F::Tables>::value,
                "Tables must be trivially constructible (it lives in shared memory)");
  static constexpr bool ok = true;
};

// ---------------------------------------------------------------------------
// Fast pipeline (nvpro_pyramid.glsl:209-534), n = 1..6.  Each CTA owns a
// 64x64 region of level L, i.e. (64 / 2^n)^2 whole reference tiles, and builds
// every level of the region in shared memory.  A tile is written only if its
// row-major index is below the coverage the dispatch's workgroup count gives
// (nvproPyramidMain assigns tile indices gl_GlobalInvocationID.x >>
// teamSizeLog2_, :414-420).
template <class F>
__global__ void __launch_bounds__(kThreads) fastKernel(const DispatchArg p) {
  static_assert(FunctorChecks<F>::ok, "");
  using V = typename F::Value;
  __shared__ typename F::Tables tables;
  __shared__ V bufA[32 * 32];
  __shared__ V bufB[16 * 16];
  F::initTables(tables, threadIdx.x, blockDim.x);
  __syncthreads();
  const F f = makeFunctors<F>(tables);

  const uint32_t n = p.n;
  const LevelArg& src = p.lv[0];
  const uint32_t tilesX = src.w >> n, tilesY = src.h >> n;
  const uint32_t coverW = tilesX << n, coverH = tilesY << n;
  const uint32_t regionsX = (coverW + kRegion - 1) / kRegion;
  const uint32_t x0 = (blockIdx.x % regionsX) * kRegion;
  const uint32_t y0 = (blockIdx.x / regionsX) * kRegion;
  const uint32_t rw = min(kRegion, coverW - x0), rh = min(kRegion, coverH - y0);
  const uint64_t tilesPerGroup = uint64_t((n > 5 ? 4096u : 1024u) >> (2 * n));
  const uint64_t limit = min(uint64_t(tilesX) * tilesY, p.groups * max(tilesPerGroup, uint64_t(1)));
  auto covered = [&](uint32_t lx, uint32_t ly) {  // level-L coordinates
    return uint64_t(ly >> n) * tilesX + (lx >> n) < limit;
  };
  const uint32_t handoff = sharedHandoffLevel(true, n);

  // Level L+1 from level L: LOAD_REDUCE4 (nvpro_pyramid.glsl:180-188).
  uint32_t ew = rw / 2, eh = rh / 2;
  for (uint32_t i = threadIdx.x; i < ew * eh; i += kThreads) {
    const uint32_t x = i % ew, y = i / ew;
    const uint32_t sx = x0 + 2 * x, sy = y0 + 2 * y;
    const V v = reduce4(f, loadAt(f, src, sx, sy), loadAt(f, src, sx, sy + 1), loadAt(f, src, sx + 1, sy),
                        loadAt(f, src, sx + 1, sy + 1));
    bufA[y * 32 + x] = handoff == 1 ? handOff(f, v) : v;
    if (covered(sx, sy)) storeAt(f, p.lv[1], x0 / 2 + x, y0 / 2 + y, v);
  }
  __syncthreads();

  V* cur = bufA;
  V* nxt = bufB;
  uint32_t curStride = 32;
  for (uint32_t k = 2; k <= n; ++k) {
    const bool vert = fastVerticalFirst(n, k);
    const uint32_t nw = ew / 2, nh = eh / 2;
    const uint32_t nStride = curStride / 2;
    for (uint32_t i = threadIdx.x; i < nw * nh; i += kThreads) {
      const uint32_t x = i % nw, y = i / nw;
      const V v = fastReduce(f, vert, cur[(2 * y) * curStride + 2 * x], cur[(2 * y) * curStride + 2 * x + 1],
                             cur[(2 * y + 1) * curStride + 2 * x], cur[(2 * y + 1) * curStride + 2 * x + 1]);
      nxt[y * nStride + x] = k == handoff ? handOff(f, v) : v;
      if (covered(x0 + (x << k), y0 + (y << k))) storeAt(f, p.lv[k], (x0 >> k) + x, (y0 >> k) + y, v);
    }
    __syncthreads();
    V* t = cur;
    cur = nxt;
    nxt = t;
    curStride = nStride;
    ew = nw;
    eh = nh;
  }
}

// ---------------------------------------------------------------------------
// General pipeline (nvpro_pyramid.glsl:536-885).

// reduceStoreSample_ (:575-656) without the store: `ld(dx, dy)` returns the
// value at offset (dx, dy) from the source corner (2x, 2y); each column is
// reduced vertically first, then the row.
template <class F, class Loader>
__device__ __forceinline__ typename F::Value reduceSample(const F& f, const Loader& ld, uint32_t kx, uint32_t ky,
                                                          uint32_t dstW, uint32_t dstH, uint32_t x, uint32_t y) {
  using V = typename F::Value;
  V h0, h1 = V(), h2 = V();
  if (ky == 3) {
    const Weights3 wy = weights3(dstH, y);
    h0 = f.reduce(wy.w0, ld(0, 0), wy.w1, ld(0, 1), wy.w2, ld(0, 2));
    if (kx >= 2) h1 = f.reduce(wy.w0, ld(1, 0), wy.w1, ld(1, 1), wy.w2, ld(1, 2));
    if (kx == 3) h2 = f.reduce(wy.w0, ld(2, 0), wy.w1, ld(2, 1), wy.w2, ld(2, 2));
  } else if (ky == 2) {
    h0 = reduce2(f, ld(0, 0), ld(0, 1));
    if (kx >= 2) h1 = reduce2(f, ld(1, 0), ld(1, 1));
    if (kx == 3) h2 = reduce2(f, ld(2, 0), ld(2, 1));
  } else {
    h0 = ld(0, 0);
    if (kx >= 2) h1 = ld(1, 0);
    if (kx == 3) h2 = ld(2, 0);
  }
  if (kx == 3) {
    const Weights3 wx = weights3(dstW, x);
    return f.reduce(wx.w0, h0, wx.w1, h1, wx.w2, h2);
  }
  if (kx == 2) return reduce2(f, h0, h1);
  return h0;
}

// One level: one thread per output texel (:828-842); workgroups of 128
// outputs in row-major order define the coverage.
template <class F>
__global__ void __launch_bounds__(kThreads) general1Kernel(const DispatchArg p) {
  static_assert(FunctorChecks<F>::ok, "");
  __shared__ typename F::Tables tables;
  F::initTables(tables, threadIdx.x, blockDim.x);
  __syncthreads();
  const F f = makeFunctors<F>(tables);
  const LevelArg &src = p.lv[0], &dst = p.lv[1];
  const uint32_t kx = kernelSize(src.w), ky = kernelSize(src.h);
  const uint64_t total = uint64_t(dst.w) * dst.h;
  const uint64_t limit = min(total, p.groups * 128u);
  for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < limit; i += uint64_t(gridDim.x) * kThreads) {
    const uint32_t x = uint32_t(i % dst.w), y = uint32_t(i / dst.w);
    auto ld = [&](uint32_t dx, uint32_t dy) { return loadAt(f, src, 2 * x + dx, 2 * y + dy); };
    storeAt(f, dst, x, y, reduceSample(f, ld, kx, ky, dst.w, dst.h, x, y));
  }
}

// Two levels: each CTA owns a 16x16 tile of level L+2 and builds the 32..33
// square window of level L+1 it needs in shared memory, as
// fillIntermediateTile_ / fillLastTile_ (:732-820) do for 8x8 tiles.  Each
// L+1 texel is stored by exactly one CTA.  Coverage follows the reference's
// 8x8 tiles: an L+2 texel is written if its 8x8 tile index is below the
// workgroup count; an L+1 texel if any such tile's 16..17 window contains it.
__device__ __forceinline__ bool g2CoveredL1(uint32_t x1, uint32_t y1, uint32_t winW, uint32_t winH,
                                            uint32_t rtilesX, uint32_t rtilesY, uint64_t groups) {
  // smallest reference 8x8-tile column / row whose window contains x1 / y1
  auto minTile = [](uint32_t c, uint32_t win, uint32_t tiles) -> int64_t {
    const uint32_t t = c / 16;
    if (win == 17 && (c % 16) == 0 && t >= 1) return t - 1;
    return t < tiles ? int64_t(t) : -1;
  };
  const int64_t tx = minTile(x1, winW, rtilesX), ty = minTile(y1, winH, rtilesY);
  if (tx < 0 || ty < 0) return false;
  return uint64_t(ty) * rtilesX + uint64_t(tx) < groups;
}

template <class F>
__global__ void __launch_bounds__(kThreads) general2Kernel(const DispatchArg p) {
  static_assert(FunctorChecks<F>::ok, "");
  using V = typename F::Value;
  __shared__ typename F::Tables tables;
  __shared__ V win[kG2Win * kG2Win];
  F::initTables(tables, threadIdx.x, blockDim.x);
  __syncthreads();
  const F f = makeFunctors<F>(tables);
  const LevelArg &l0 = p.lv[0], &l1 = p.lv[1], &l2 = p.lv[2];
  const uint32_t kx = kernelSize(l0.w), ky = kernelSize(l0.h);
  const uint32_t fkx = kernelSize(l1.w), fky = kernelSize(l1.h);
  const uint32_t tilesX = (l2.w + kG2Tile - 1) / kG2Tile, tilesY = (l2.h + kG2Tile - 1) / kG2Tile;
  const uint32_t tx = blockIdx.x % tilesX, ty = blockIdx.x / tilesX;
  const uint32_t rtilesX = (l2.w + 7) / 8, rtilesY = (l2.h + 7) / 8;
  const bool full = p.groups >= uint64_t(rtilesX) * rtilesY;
  const uint32_t refWinW = fkx == 3 ? 17 : 16, refWinH = fky == 3 ? 17 : 16;

  const uint32_t wx0 = tx * 2 * kG2Tile, wy0 = ty * 2 * kG2Tile;
  const uint32_t ww = min(2 * kG2Tile + (fkx == 3), l1.w - wx0);
  const uint32_t wh = min(2 * kG2Tile + (fky == 3), l1.h - wy0);
  for (uint32_t i = threadIdx.x; i < ww * wh; i += kThreads) {
    const uint32_t wx = i % ww, wy = i / ww;
    const uint32_t x = wx0 + wx, y = wy0 + wy;
    auto ld = [&](uint32_t dx, uint32_t dy) { return loadAt(f, l0, 2 * x + dx, 2 * y + dy); };
    const V v = reduceSample(f, ld, kx, ky, l1.w, l1.h, x, y);
    win[wy * kG2Win + wx] = handOff(f, v);  // level L+1 is the hand-off level of a two-level dispatch
    const bool owner = min(x / (2 * kG2Tile), tilesX - 1) == tx && min(y / (2 * kG2Tile), tilesY - 1) == ty;
    if (owner && (full || g2CoveredL1(x, y, refWinW, refWinH, rtilesX, rtilesY, p.groups))) storeAt(f, l1, x, y, v);
  }
  __syncthreads();
  const uint32_t lx = threadIdx.x % kG2Tile, ly = threadIdx.x / kG2Tile;
  const uint32_t x = tx * kG2Tile + lx, y = ty * kG2Tile + ly;
  if (x < l2.w && y < l2.h && (full || uint64_t(y / 8) * rtilesX + x / 8 < p.groups)) {
    auto ld = [&](uint32_t dx, uint32_t dy) { return win[(2 * ly + dy) * kG2Win + 2 * lx + dx]; };
    storeAt(f, l2, x, y, reduceSample(f, ld, fkx, fky, l2.w, l2.h, x, y));
  }
}

// Launch the kernel of one dispatch of `images` images (grid z).
template <class F>
cudaError_t launchDispatch(const DispatchArg& p, uint32_t images, cudaStream_t stream, uint32_t* launches) {
  if (images == 0 || images > 65535) return cudaErrorInvalidValue;
  if (p.isFast) {
    const uint32_t n = p.n;
    const uint32_t coverW = (p.lv[0].w >> n) << n, coverH = (p.lv[0].h >> n) << n;
    const uint64_t regions = uint64_t((coverW + kRegion - 1) / kRegion) * ((coverH + kRegion - 1) / kRegion);
    if (regions == 0 || p.groups == 0) return cudaSuccess;
    fastKernel<F><<<dim3(uint32_t(regions), 1, images), kThreads, 0, stream>>>(p);
  } else if (p.n == 1) {
    const uint64_t total = uint64_t(p.lv[1].w) * p.lv[1].h;
    const uint64_t work = total < p.groups * 128u ? total : p.groups * 128u;
    if (work == 0) return cudaSuccess;
    const uint64_t blocks = (work + kThreads - 1) / kThreads;
    general1Kernel<F><<<dim3(uint32_t(blocks < 152u * 64u ? blocks : 152u * 64u), 1, images), kThreads, 0, stream>>>(p);
  } else {
    const uint64_t tiles = uint64_t((p.lv[2].w + kG2Tile - 1) / kG2Tile) * ((p.lv[2].h + kG2Tile - 1) / kG2Tile);
    if (p.groups == 0) return cudaSuccess;
    general2Kernel<F><<<dim3(uint32_t(tiles), 1, images), kThreads, 0, stream>>>(p);
  }
  ++*launches;
  return cudaGetLastError();
}

// The launcher of a pipeline of F (nvpro_pyramid_launcher_t).
template <class F>
NvproPyramidResult launchCustom(void* /*userData*/, NvproPyramidStream stream, const NvproPyramidDispatchDesc* d) {
  if (!d || d->levelCount < 1 || d->levelCount > 6 || (!d->isFastPipeline && d->levelCount > 2))
    return NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT;
  DispatchArg a{};
  a.isFast = d->isFastPipeline;
  a.n = d->levelCount;
  a.groups = d->groupCount;
  for (uint32_t k = 0; k <= d->levelCount; ++k) {
    const NvproPyramidLevelDesc& l = d->levels[k];
    a.lv[k] = LevelArg{static_cast<uint8_t*>(l.texels), l.rowPitchBytes, l.width, l.height, l.imageStrideBytes};
  }
  uint32_t launches = 0;
  const cudaError_t e = launchDispatch<F>(a, d->imageCount, reinterpret_cast<cudaStream_t>(stream), &launches);
  return e == cudaSuccess ? NVPRO_PYRAMID_SUCCESS : NVPRO_PYRAMID_ERROR_CUDA;
}

}  // namespace detail

/* The general pipeline of F (and its fast pipeline, if `fast` is not NULL)
 * as NvproPyramidPipeline handles for nvproCmdPyramidDispatch /
 * nvproPyramidGenerate: the vkCreateComputePipelines of a shader that defines
 * the customisation macros (minimal_app/minimal_mipmaps.cpp:178-190).
 * Destroy them with nvproPyramidDestroyPipeline. */
template <class F>
NvproPyramidResult createPipelines(NvproPyramidPipeline* general, NvproPyramidPipeline* fast = nullptr) {
  if (!general) return NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT;
  const uint32_t bytes = uint32_t(sizeof(typename F::Texel));
  NvproPyramidResult r = nvproPyramidCreateCustomPipeline(0, bytes, &detail::launchCustom<F>, nullptr, general);
  if (r == NVPRO_PYRAMID_SUCCESS && fast) {
    r = nvproPyramidCreateCustomPipeline(1, bytes, &detail::launchCustom<F>, nullptr, fast);
    if (r != NVPRO_PYRAMID_SUCCESS) {
      nvproPyramidDestroyPipeline(*general);
      *general = nullptr;
    }
  }
  return r;
}

}  // namespace nvpro_pyramid

#endif /* NVPRO_PYRAMID_CUDA_HPP_ */
