// kernels_portable.cu -- the fast and general pyramid pipelines for any
// preset and any level layout (per-level pointers and row pitches), with plain
// global loads and stores.  These kernels define the library's semantics; the
// TMA kernels (kernels_tma.cu) are faster equivalents for aligned layouts and
// produce identical bytes.
//
// Semantics follow nvpro_pyramid.glsl dispatch by dispatch: a fast dispatch of
// n levels reduces each 2^n x 2^n tile of level L with 2x2 box filters whose
// operand order is fastVerticalFirst(n, k); a general dispatch of 1 or 2 levels
// applies the 1..3-tap energy-conserving kernel.  Values stay FP32 inside a
// dispatch and are quantised only by the STORE of each level, except the
// hand-off level of a pipeline with a shared-memory format (handOff).
#include <algorithm>

#include "device_common.cuh"

namespace nvpyr {
namespace {

constexpr uint32_t kRegion = 64;  // fast kernels: 64x64 region of level L per CTA
constexpr uint32_t kThreads = 256;

template <uint32_t P>
struct SmemTables {
  SrgbTablesSmem t;
};

// Level L+k of this CTA's image (blockIdx.z of a strided batch).
__device__ __forceinline__ LevelView levelOf(const DispatchParams& p, uint32_t k) {
  LevelView v = p.lv[k];
  v.ptr += uint64_t(blockIdx.z) * p.imageStride[k];
  return v;
}

template <uint32_t P>
__device__ __forceinline__ TexelIO<P> makeIO(SrgbTablesSmem* t) {
  TexelIO<P> io;
  io.t = t;
  return io;
}

// The value a dispatch hands on to its next level through the reference's
// shared memory, in the pipeline's shared format `fmt` (sRGBA8 only;
// srgba8_mipmap_preamble.glsl:60-108): the texel's code decoded again, or
// each channel as binary16.  The hand-off level itself is stored from v.
template <uint32_t P>
__device__ __forceinline__ float4 handOff(uint32_t fmt, float4 v, const TexelIO<P>& io) {
  if constexpr (P == kSrgba8) {
    if (fmt == kSharedSrgb) return io.decode(io.encode(v));
    if (fmt == kSharedF16) return f16RoundTrip(v);
  }
  return v;
}

// ---------------------------------------------------------------------------
// Fast pipeline (nvpro_pyramid.glsl:209-534), n = 1..6.
//
// Each CTA owns a 64x64 region of level L, i.e. (64 / 2^n)^2 whole reference
// tiles, and builds every level of the region in shared memory.  A tile is
// written only if its row-major index is below the coverage limit implied by
// the dispatch's workgroup count (nvproPyramidMain assigns tile indices
// gl_GlobalInvocationID.x >> teamSizeLog2_, :414-420).
template <uint32_t P>
__global__ void __launch_bounds__(kThreads) portableFastKernel(DispatchParams p) {
  __shared__ SrgbTablesSmem tabs;
  __shared__ float4 bufA[32 * 32];
  __shared__ float4 bufB[16 * 16];
  if (P == kSrgba8) {
    loadSrgbTables(&tabs);
    __syncthreads();
  }
  const TexelIO<P> io = makeIO<P>(&tabs);
  constexpr uint32_t B = TexelIO<P>::kBytes;

  const uint32_t n = p.levelCount;
  const LevelView src = levelOf(p, 0);
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

  // Level L+1 from global level L: LOAD_REDUCE4 (nvpro_pyramid.glsl:180-188).
  const LevelView dst1 = levelOf(p, 1);
  uint32_t ew = rw / 2, eh = rh / 2;
  for (uint32_t i = threadIdx.x; i < ew * eh; i += kThreads) {
    const uint32_t x = i % ew, y = i / ew;
    const uint32_t sx = x0 + 2 * x, sy = y0 + 2 * y;
    const float4 v00 = io.load(texelAddr(src, sx, sy, B));
    const float4 v01 = io.load(texelAddr(src, sx, sy + 1, B));
    const float4 v10 = io.load(texelAddr(src, sx + 1, sy, B));
    const float4 v11 = io.load(texelAddr(src, sx + 1, sy + 1, B));
    const float4 v = reduce4(v00, v01, v10, v11);
    bufA[y * 32 + x] = v;
    if (covered(sx, sy)) io.store(texelAddr(dst1, x0 / 2 + x, y0 / 2 + y, B), v);
  }
  __syncthreads();

  float4* cur = bufA;
  float4* nxt = bufB;
  uint32_t curStride = 32;
  const uint32_t handoffLevel = p.sharedFmt != kSharedFp32 ? sharedHandoffLevel(true, n) : 0u;
  for (uint32_t k = 2; k <= n; ++k) {
    const bool vert = fastVerticalFirst(n, k);
    const uint32_t nw = ew / 2, nh = eh / 2;
    const uint32_t nStride = curStride / 2;
    for (uint32_t i = threadIdx.x; i < nw * nh; i += kThreads) {
      const uint32_t x = i % nw, y = i / nw;
      const float4 tl = cur[(2 * y) * curStride + 2 * x], tr = cur[(2 * y) * curStride + 2 * x + 1];
      const float4 bl = cur[(2 * y + 1) * curStride + 2 * x], br = cur[(2 * y + 1) * curStride + 2 * x + 1];
      const float4 v = fastReduce(vert, tl, tr, bl, br);
      nxt[y * nStride + x] = k == handoffLevel ? handOff<P>(p.sharedFmt, v, io) : v;
      if (covered(x0 + (x << k), y0 + (y << k)))
        io.store(texelAddr(levelOf(p, k), (x0 >> k) + x, (y0 >> k) + y, B), v);
    }
    __syncthreads();
    float4* t = cur;
    cur = nxt;
    nxt = t;
    curStride = nStride;
    ew = nw;
    eh = nh;
  }
}

// ---------------------------------------------------------------------------
// General pipeline (nvpro_pyramid.glsl:536-885).

// reduceStoreSample_ (:575-656) without the store; `ld(dx, dy)` returns the
// FP32 sample at offset (dx, dy) from the source corner (2x, 2y).
template <typename Loader>
__device__ __forceinline__ float4 reduceSample(const Loader& ld, uint32_t kx, uint32_t ky, uint32_t dstW,
                                               uint32_t dstH, uint32_t x, uint32_t y) {
  float4 h0, h1 = make_float4(0, 0, 0, 0), h2 = make_float4(0, 0, 0, 0);
  if (ky == 3) {
    const Weights3 wy = weights3(dstH, y);
    h0 = reduce3(wy.w0, ld(0, 0), wy.w1, ld(0, 1), wy.w2, ld(0, 2));
    if (kx >= 2) h1 = reduce3(wy.w0, ld(1, 0), wy.w1, ld(1, 1), wy.w2, ld(1, 2));
    if (kx == 3) h2 = reduce3(wy.w0, ld(2, 0), wy.w1, ld(2, 1), wy.w2, ld(2, 2));
  } else if (ky == 2) {
    h0 = reduce2(ld(0, 0), ld(0, 1));
    if (kx >= 2) h1 = reduce2(ld(1, 0), ld(1, 1));
    if (kx == 3) h2 = reduce2(ld(2, 0), ld(2, 1));
  } else {
    h0 = ld(0, 0);
    if (kx >= 2) h1 = ld(1, 0);
    if (kx == 3) h2 = ld(2, 0);
  }
  if (kx == 3) {
    const Weights3 wx = weights3(dstW, x);
    return reduce3(wx.w0, h0, wx.w1, h1, wx.w2, h2);
  }
  if (kx == 2) return reduce2(h0, h1);
  return h0;
}

// One level: one thread per output texel (:828-842); workgroups of 128
// outputs in row-major order define the coverage limit.
template <uint32_t P>
__global__ void __launch_bounds__(kThreads) portableGeneral1Kernel(DispatchParams p) {
  __shared__ SrgbTablesSmem tabs;
  if (P == kSrgba8) {
    loadSrgbTables(&tabs);
    __syncthreads();
  }
  const TexelIO<P> io = makeIO<P>(&tabs);
  constexpr uint32_t B = TexelIO<P>::kBytes;
  const LevelView src = levelOf(p, 0);
  const LevelView dst = levelOf(p, 1);
  const uint32_t kx = kernelSize(src.w), ky = kernelSize(src.h);
  const uint64_t total = uint64_t(dst.w) * dst.h;
  const uint64_t limit = min(total, p.groups * 128u);
  for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < limit; i += uint64_t(gridDim.x) * kThreads) {
    const uint32_t x = uint32_t(i % dst.w), y = uint32_t(i / dst.w);
    auto ld = [&](uint32_t dx, uint32_t dy) { return io.load(texelAddr(src, 2 * x + dx, 2 * y + dy, B)); };
    io.store(texelAddr(dst, x, y, B), reduceSample(ld, kx, ky, dst.w, dst.h, x, y));
  }
}

// Two levels: each CTA owns a 16x16 tile of level L+2 and builds the 32..33
// square window of level L+1 it needs in shared memory (FP32), as
// fillIntermediateTile_/fillLastTile_ (:732-820) do for 8x8 tiles.  Each L+1
// texel is stored by exactly one CTA.  Coverage follows the reference's 8x8
// tiles: an L+2 texel is written if its 8x8 tile index is below the workgroup
// count; an L+1 texel if any such tile's 16..17 window contains it.
constexpr uint32_t kG2Tile = 16;
constexpr uint32_t kG2Win = 2 * kG2Tile + 1;

__device__ __forceinline__ bool g2CoveredL1(uint32_t x1, uint32_t y1, uint32_t winW, uint32_t winH,
                                            uint32_t rtilesX, uint32_t rtilesY, uint64_t groups) {
  // Smallest reference 8x8-tile column / row whose window contains x1 / y1.
  auto minTile = [](uint32_t c, uint32_t win, uint32_t tiles) -> int64_t {
    const uint32_t t = c / 16;
    if (win == 17 && (c % 16) == 0 && t >= 1) return t - 1;
    return t < tiles ? int64_t(t) : -1;
  };
  const int64_t tx = minTile(x1, winW, rtilesX), ty = minTile(y1, winH, rtilesY);
  if (tx < 0 || ty < 0) return false;
  return uint64_t(ty) * rtilesX + uint64_t(tx) < groups;
}

template <uint32_t P>
__global__ void __launch_bounds__(kThreads) portableGeneral2Kernel(DispatchParams p) {
  __shared__ SrgbTablesSmem tabs;
  __shared__ float4 win[kG2Win * kG2Win];
  if (P == kSrgba8) loadSrgbTables(&tabs);
  __syncthreads();
  const TexelIO<P> io = makeIO<P>(&tabs);
  constexpr uint32_t B = TexelIO<P>::kBytes;
  const LevelView l0 = levelOf(p, 0);
  const LevelView l1 = levelOf(p, 1);
  const LevelView l2 = levelOf(p, 2);
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
    auto ld = [&](uint32_t dx, uint32_t dy) { return io.load(texelAddr(l0, 2 * x + dx, 2 * y + dy, B)); };
    const float4 v = reduceSample(ld, kx, ky, l1.w, l1.h, x, y);
    win[wy * kG2Win + wx] = handOff<P>(p.sharedFmt, v, io);
    const bool owner = min(x / (2 * kG2Tile), tilesX - 1) == tx && min(y / (2 * kG2Tile), tilesY - 1) == ty;
    if (owner && (full || g2CoveredL1(x, y, refWinW, refWinH, rtilesX, rtilesY, p.groups)))
      io.store(texelAddr(l1, x, y, B), v);
  }
  __syncthreads();
  {
    const uint32_t lx = threadIdx.x % kG2Tile, ly = threadIdx.x / kG2Tile;
    const uint32_t x = tx * kG2Tile + lx, y = ty * kG2Tile + ly;
    if (x < l2.w && y < l2.h && (full || uint64_t(y / 8) * rtilesX + x / 8 < p.groups)) {
      auto ld = [&](uint32_t dx, uint32_t dy) { return win[(2 * ly + dy) * kG2Win + 2 * lx + dx]; };
      io.store(texelAddr(l2, x, y, B), reduceSample(ld, fkx, fky, l2.w, l2.h, x, y));
    }
  }
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
  const TexelIO<P> io = makeIO<P>(&tabs);
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
cudaError_t launchPreset(const DispatchParams& p, cudaStream_t stream, uint32_t* launches) {
  if (p.isBlit) {
    const uint64_t total = uint64_t(p.lv[1].w) * p.lv[1].h;
    const uint64_t blocks = std::min<uint64_t>((total + kThreads - 1) / kThreads, 152u * 64u);
    portableBlitKernel<P><<<dim3(uint32_t(blocks), 1, p.batch), kThreads, 0, stream>>>(p);
  } else if (p.isFast) {
    const uint32_t n = p.levelCount;
    const uint32_t coverW = (p.lv[0].w >> n) << n, coverH = (p.lv[0].h >> n) << n;
    const uint64_t regions = uint64_t((coverW + kRegion - 1) / kRegion) * ((coverH + kRegion - 1) / kRegion);
    if (regions == 0 || p.groups == 0) return cudaSuccess;
    portableFastKernel<P><<<dim3(uint32_t(regions), 1, p.batch), kThreads, 0, stream>>>(p);
  } else if (p.levelCount == 1) {
    const uint64_t total = uint64_t(p.lv[1].w) * p.lv[1].h;
    const uint64_t work = std::min<uint64_t>(total, p.groups * 128u);
    if (work == 0) return cudaSuccess;
    const uint64_t blocks = std::min<uint64_t>((work + kThreads - 1) / kThreads, 152u * 64u);
    portableGeneral1Kernel<P><<<dim3(uint32_t(blocks), 1, p.batch), kThreads, 0, stream>>>(p);
  } else {
    const uint64_t tiles = uint64_t((p.lv[2].w + kG2Tile - 1) / kG2Tile) * ((p.lv[2].h + kG2Tile - 1) / kG2Tile);
    if (p.groups == 0) return cudaSuccess;
    portableGeneral2Kernel<P><<<dim3(uint32_t(tiles), 1, p.batch), kThreads, 0, stream>>>(p);
  }
  ++*launches;
  return cudaGetLastError();
}

}  // namespace

cudaError_t launchPortable(const DispatchParams& p, cudaStream_t stream, uint32_t* launches) {
  switch (p.preset) {
    case kSrgba8:
      return launchPreset<kSrgba8>(p, stream, launches);
    case kRgba32f:
      return launchPreset<kRgba32f>(p, stream, launches);
    case kRgba16f:
      return launchPreset<kRgba16f>(p, stream, launches);
  }
  return cudaErrorInvalidValue;
}

}  // namespace nvpyr
