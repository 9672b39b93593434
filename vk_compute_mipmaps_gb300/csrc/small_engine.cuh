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
// code buffers: the input level of the run (kSmallMaxTexels codes, loaded from
// global memory at the start) and the output level of a dispatch, which
// alternate between dispatches.  A dispatch fits if level L+1 has at most
// kSmallL1Texels texels and level L+2 at most kSmallL2Texels (always, for
// levels at least four texels on each side; see smallDispatchFits).
constexpr uint32_t kSmallL1Texels = kSmallMaxTexels / 4;
constexpr uint32_t kSmallL2Texels = kSmallMaxTexels / 16;
constexpr uint32_t kSmallArenaBytes = 16 * (kSmallL1Texels + kSmallL2Texels) + 4 * (kSmallMaxTexels + kSmallL1Texels);

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

// floor(t / w) for t < 2^20 as a multiply-high by r = recip32(w) = floor((2^32 - 1) / w) + 1:
// t * r / 2^32 exceeds t / w by less than t / 2^32, less than the distance to the next integer.
__device__ __forceinline__ uint32_t recip32(uint32_t w) { return 0xFFFFFFFFu / w + 1u; }
__device__ __forceinline__ uint32_t divBy(uint32_t t, uint32_t r, uint32_t w) {
  return w == 1 ? t : __umulhi(t, r);
}

// Input texel (x, y) of a level step: a stored code (decoded) or an FP32
// value handed on inside the dispatch.
template <bool CODES, typename Codec>
__device__ __forceinline__ float4 smallIn(const uint32_t* codes, const float4* vals, uint32_t w, uint32_t x,
                                          uint32_t y, const Codec& C) {
  return CODES ? C.decode(codes[y * w + x]) : vals[y * w + x];
}

// One level of a dispatch: level k (wk x hk) from level k-1 (wi x hi), every
// texel stored to global memory, and kept as a code (last level of the
// dispatch) or as an FP32 value (after the shared format at the hand-off level).
template <bool CODES, bool FAST, typename Codec>
__device__ __forceinline__ void smallLevel(const uint32_t* inCodes, const float4* inVals, uint32_t wi, uint32_t hi,
                                           uint32_t wk, uint32_t hk, bool vert, uint8_t* dst, uint64_t pitch,
                                           uint32_t* outCodes, float4* outVals, bool handoff, uint32_t sharedFmt,
                                           const Codec& C, uint32_t tid, uint32_t nthreads) {
  const uint32_t kx = kernelSize(wi), ky = kernelSize(hi);
  const uint32_t r = recip32(wk);
  // the 3-tap weights with 1 / (2n + 1) computed once per level (weights3's
  // arithmetic, term by term)
  const float nfx = __uint2float_rn(wk), nfy = __uint2float_rn(hk);
  const float rcpx = __frcp_rn(__fadd_rn(__fmul_rn(2.0f, nfx), 1.0f));
  const float rcpy = __frcp_rn(__fadd_rn(__fmul_rn(2.0f, nfy), 1.0f));
  auto wts = [](float nf, float rcp, uint32_t i) {
    Weights3 w;
    w.w0 = __fmul_rn(rcp, __fsub_rn(nf, __uint2float_rn(i)));
    w.w1 = __fmul_rn(rcp, nf);
    w.w2 = __fsub_rn(__fsub_rn(1.0f, w.w0), w.w1);
    return w;
  };
  // Not unrolled: the engine runs once per launch in one CTA, where the
  // shorter code is worth more than the overlap of two texels (measured:
  // 4096^2 chain 43.4 -> 42.2 us, 2560x1440 42.1 -> 39.3 us per launch).
#pragma unroll 1
  for (uint32_t t = tid; t < wk * hk; t += nthreads) {
    const uint32_t y = divBy(t, r, wk), x = t - y * wk;
    float4 v;
    if (FAST) {
      const float4 tl = smallIn<CODES>(inCodes, inVals, wi, 2 * x, 2 * y, C);
      const float4 tr = smallIn<CODES>(inCodes, inVals, wi, 2 * x + 1, 2 * y, C);
      const float4 bl = smallIn<CODES>(inCodes, inVals, wi, 2 * x, 2 * y + 1, C);
      const float4 br = smallIn<CODES>(inCodes, inVals, wi, 2 * x + 1, 2 * y + 1, C);
      v = fastReduce(vert, tl, tr, bl, br);
    } else {
      // kernel size 1 reads row / column 0 only; 2 and 3 their taps
      const uint32_t y1 = ky > 1 ? 2 * y + 1 : 2 * y, y2 = ky > 2 ? 2 * y + 2 : 2 * y;
      const Weights3 wy = wts(nfy, rcpy, y);
      float4 h[3];
#pragma unroll
      for (uint32_t c = 0; c < 3; ++c) {
        const uint32_t xc = 2 * x + (c < kx ? c : 0);
        const float4 a = smallIn<CODES>(inCodes, inVals, wi, xc, 2 * y, C);
        const float4 b = smallIn<CODES>(inCodes, inVals, wi, xc, y1, C);
        const float4 e = smallIn<CODES>(inCodes, inVals, wi, xc, y2, C);
        h[c] = ky == 3 ? reduce3(wy.w0, a, wy.w1, b, wy.w2, e) : ky == 2 ? reduce2(a, b) : a;
      }
      if (kx == 3) {
        const Weights3 wx = wts(nfx, rcpx, x);
        v = reduce3(wx.w0, h[0], wx.w1, h[1], wx.w2, h[2]);
      } else {
        v = kx == 2 ? reduce2(h[0], h[1]) : h[0];
      }
    }
    const uint32_t code = C.encode(v);
    *reinterpret_cast<uint32_t*>(dst + uint64_t(y) * pitch + uint64_t(x) * 4) = code;
    if (outCodes) {
      outCodes[t] = code;
    } else {
      if (handoff) {
        if (sharedFmt == kSharedSrgb) v = C.decode(code);
        else if (sharedFmt == kSharedF16) v = f16RoundTrip(v);
      }
      outVals[t] = v;
    }
  }
}

template <typename Codec>
__device__ __forceinline__ void runSmallDispatches(const SmallDispatch* ds, uint32_t count, uint8_t* arena,
                                                const Codec C, uint32_t tid, uint32_t nthreads) {
  float4* const bufA = reinterpret_cast<float4*>(arena);
  float4* const bufB = bufA + kSmallL1Texels;
  uint32_t* const codesIn = reinterpret_cast<uint32_t*>(bufB + kSmallL2Texels);  // kSmallMaxTexels
  uint32_t* const codesOut = codesIn + kSmallMaxTexels;                          // kSmallL1Texels
  // The run's input level into shared memory, eight loads in flight per thread.
  {
    const uint32_t w0 = ds[0].w0, n0 = w0 * ds[0].h0, r0 = recip32(w0);
    const uint8_t* const src = ds[0].src;
    const uint64_t srcPitch = ds[0].srcPitch;
    for (uint32_t t0 = tid; t0 < n0; t0 += 8 * nthreads) {
      uint32_t v[8];
#pragma unroll
      for (uint32_t j = 0; j < 8; ++j) {
        const uint32_t t = t0 + j * nthreads;
        if (t < n0) {
          const uint32_t y = divBy(t, r0, w0);
          v[j] = ldcgTexel(src + uint64_t(y) * srcPitch + uint64_t(t - y * w0) * 4);
        }
      }
#pragma unroll
      for (uint32_t j = 0; j < 8; ++j)
        if (t0 + j * nthreads < n0) codesIn[t0 + j * nthreads] = v[j];
    }
  }
  __syncthreads();
  // the input codes of dispatch i, its output codes (they alternate)
  uint32_t* in = codesIn;
  uint32_t* out = codesOut;
#pragma unroll 1
  for (uint32_t i = 0; i < count; ++i) {
    const uint32_t isFast = ds[i].isFast, n = ds[i].n, sharedFmt = ds[i].sharedFmt;
    const uint32_t handoff = sharedHandoffLevel(isFast != 0, n);
    uint32_t wi = ds[i].w0, hi = ds[i].h0;
#pragma unroll 1
    for (uint32_t k = 1; k <= n; ++k) {
      const uint32_t wk = max(wi >> 1, 1u), hk = max(hi >> 1, 1u);
      float4* const outVals = k < n ? ((k & 1) ? bufA : bufB) : nullptr;
      const float4* const inVals = (k & 1) ? bufB : bufA;  // level k-1's values (k >= 2)
      uint32_t* const outCodes = k == n ? out : nullptr;
      const bool vert = fastVerticalFirst(n, k);
      uint8_t* const dst = ds[i].dst[k - 1];
      const uint64_t pitch = ds[i].pitch[k - 1];
      if (k == 1) {
        if (isFast)
          smallLevel<true, true>(in, inVals, wi, hi, wk, hk, vert, dst, pitch, outCodes, outVals, k == handoff,
                                 sharedFmt, C, tid, nthreads);
        else
          smallLevel<true, false>(in, inVals, wi, hi, wk, hk, vert, dst, pitch, outCodes, outVals, k == handoff,
                                  sharedFmt, C, tid, nthreads);
      } else {
        if (isFast)
          smallLevel<false, true>(in, inVals, wi, hi, wk, hk, vert, dst, pitch, outCodes, outVals, k == handoff,
                                  sharedFmt, C, tid, nthreads);
        else
          smallLevel<false, false>(in, inVals, wi, hi, wk, hk, vert, dst, pitch, outCodes, outVals,
                                   k == handoff, sharedFmt, C, tid, nthreads);
      }
      __syncthreads();
      wi = wk;
      hi = hk;
    }
    uint32_t* const t = in;  // swap: this output is the next input (later levels fit either buffer)
    in = out;
    out = t;
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
