// small_engine.cuh -- dispatches on small levels, run by one CTA with all its
// threads: the trailing dispatches of a chain (after the launch's large
// dispatch, the last CTA to finish runs them) and whole chains of small
// images.  Any sRGBA8 dispatch whose input level has at most kSmallMaxTexels
// texels: fast (nvpro_pyramid.glsl:229-532) or general (:550-882), including
// levels one texel wide.
//
// A dispatch is computed level by level.  Each thread takes output texels
// t, t + nthreads, ... of the level; a __syncthreads separates levels.  The
// values handed from one level to the next inside a dispatch stay FP32 in
// shared memory (after the pipeline's shared format at the hand-off level,
// nvpro_pyramid.glsl:253,555 with srgba8_mipmap_preamble.glsl:60-108); the
// last level of a dispatch is stored, and its codes are also kept in shared
// memory as the next dispatch's input, which is exactly what that dispatch
// would read back.  Only the first dispatch reads its input from global
// memory (L2-coherent loads: other CTAs of the launch wrote it).  Every texel
// is reduced with the operation order of the per-dispatch kernels, so the
// bytes equal them and the oracle: fast levels in the order of
// fastVerticalFirst(n, k), general levels vertical first per column, then
// horizontal (reduceStoreSample_, :575-656).
#pragma once
#include "srgb_codec.cuh"

namespace nvpyr {

// One dispatch for the engine.
struct SmallDispatch {
  uint32_t isFast, n, sharedFmt;
  uint32_t w0, h0;     // input level
  const uint8_t* src;  // input level (read by the first dispatch of a run only)
  uint64_t srcPitch;
  uint8_t* dst[kMaxDispatchLevels];  // levels L+1 .. L+n
  uint64_t pitch[kMaxDispatchLevels];
};

// Shared memory of the engine: FP32 levels L+1 and L+2 of a dispatch, and two
// code buffers (the output level of the previous dispatch, of this one).  A
// dispatch fits if level L+1 has at most kSmallL1Texels texels and level L+2
// at most kSmallL2Texels (always, for levels at least four texels on each
// side; see smallDispatchFits).
constexpr uint32_t kSmallL1Texels = kSmallMaxTexels / 4;
constexpr uint32_t kSmallL2Texels = kSmallMaxTexels / 16;
constexpr uint32_t kSmallArenaBytes = 16 * (kSmallL1Texels + kSmallL2Texels) + 2 * 4 * kSmallL1Texels;

// The sRGB codec through the replicated tables of a Lut made by makeLutAt
// (the TMA kernel's layout).
struct LutCodec {
  Lut L;
  __device__ __forceinline__ float4 decode(uint32_t w) const { return decodeTexel(w, L); }
  __device__ __forceinline__ uint32_t encode(float4 v) const { return encodeTexel(v, L); }
};

__device__ __forceinline__ uint32_t ldcgTexel(const uint8_t* p) {
  return __ldcg(reinterpret_cast<const unsigned int*>(p));
}

template <typename Codec>
__device__ __noinline__ void runSmallDispatches(const SmallDispatch* ds, uint32_t count, uint8_t* arena,
                                                const Codec& C, uint32_t tid, uint32_t nthreads) {
  float4* const bufA = reinterpret_cast<float4*>(arena);
  float4* const bufB = bufA + kSmallL1Texels;
  uint32_t* const codes0 = reinterpret_cast<uint32_t*>(bufB + kSmallL2Texels);
  uint32_t* const codes1 = codes0 + kSmallL1Texels;
  const uint32_t* inCodes = nullptr;  // output codes of the previous dispatch
#pragma unroll 1
  for (uint32_t i = 0; i < count; ++i) {
    const SmallDispatch d = ds[i];
    const uint32_t handoff = sharedHandoffLevel(d.isFast != 0, d.n);
    uint32_t* const outCodes = (i & 1) ? codes1 : codes0;
    uint32_t wi = d.w0, hi = d.h0;
    const float4* inF = nullptr;
#pragma unroll 1
    for (uint32_t k = 1; k <= d.n; ++k) {
      const uint32_t wk = max(wi >> 1, 1u), hk = max(hi >> 1, 1u);
      float4* const outF = k < d.n ? ((k & 1) ? bufA : bufB) : nullptr;
      const uint32_t kx = kernelSize(wi), ky = kernelSize(hi);
      const bool vert = fastVerticalFirst(d.n, k);
      uint8_t* const dst = d.dst[k - 1];
      const uint64_t pitch = d.pitch[k - 1];
      auto in = [&](uint32_t x, uint32_t y) -> float4 {
        if (inF) return inF[y * wi + x];
        return C.decode(inCodes ? inCodes[y * wi + x]
                                : ldcgTexel(d.src + uint64_t(y) * d.srcPitch + uint64_t(x) * 4));
      };
      for (uint32_t t = tid; t < wk * hk; t += nthreads) {
        const uint32_t x = t % wk, y = t / wk;
        float4 v;
        if (d.isFast) {
          v = fastReduce(vert, in(2 * x, 2 * y), in(2 * x + 1, 2 * y), in(2 * x, 2 * y + 1),
                         in(2 * x + 1, 2 * y + 1));
        } else {
          float4 h[3];
#pragma unroll
          for (uint32_t c = 0; c < 3; ++c) {
            if (c >= kx) break;
            if (ky == 3) {
              const Weights3 w = weights3(hk, y);
              h[c] = reduce3(w.w0, in(2 * x + c, 2 * y), w.w1, in(2 * x + c, 2 * y + 1), w.w2,
                             in(2 * x + c, 2 * y + 2));
            } else if (ky == 2) {
              h[c] = reduce2(in(2 * x + c, 2 * y), in(2 * x + c, 2 * y + 1));
            } else {
              h[c] = in(2 * x + c, 2 * y);
            }
          }
          if (kx == 3) {
            const Weights3 w = weights3(wk, x);
            v = reduce3(w.w0, h[0], w.w1, h[1], w.w2, h[2]);
          } else if (kx == 2) {
            v = reduce2(h[0], h[1]);
          } else {
            v = h[0];
          }
        }
        const uint32_t code = C.encode(v);
        *reinterpret_cast<uint32_t*>(dst + uint64_t(y) * pitch + uint64_t(x) * 4) = code;
        if (k == d.n) {
          outCodes[t] = code;
        } else {
          if (k == handoff) {
            if (d.sharedFmt == kSharedSrgb) v = C.decode(code);
            else if (d.sharedFmt == kSharedF16) v = f16RoundTrip(v);
          }
          outF[t] = v;
        }
      }
      __syncthreads();
      inF = outF;
      wi = wk;
      hi = hk;
    }
    inCodes = outCodes;
  }
}

// Host side: the sizes of a dispatch fit the engine's buffers.
inline bool smallDispatchFits(const DispatchParams& p) {
  auto texels = [&](uint32_t k) {
    const uint32_t w = p.lv[0].w >> k, h = p.lv[0].h >> k;
    return uint64_t(w ? w : 1) * (h ? h : 1);
  };
  return texels(0) <= kSmallMaxTexels && texels(1) <= kSmallL1Texels &&
         (p.levelCount < 3 || texels(2) <= kSmallL2Texels);
}

inline void makeSmallDispatch(const DispatchParams& p, SmallDispatch* d) {
  *d = SmallDispatch{};
  d->isFast = p.isFast;
  d->n = p.levelCount;
  d->sharedFmt = p.sharedFmt;
  d->w0 = p.lv[0].w;
  d->h0 = p.lv[0].h;
  d->src = p.lv[0].ptr;
  d->srcPitch = p.lv[0].pitch;
  for (uint32_t k = 1; k <= p.levelCount; ++k) {
    d->dst[k - 1] = p.lv[k].ptr;
    d->pitch[k - 1] = p.lv[k].pitch;
  }
}

}  // namespace nvpyr
