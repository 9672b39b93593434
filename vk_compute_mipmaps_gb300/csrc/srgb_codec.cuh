// srgb_codec.cuh -- the sRGBA8 codec of the fast kernels and the packed
// FP32 reduction helpers they share.
//
// Decode is a table lookup per channel from a table replicated once per lane
// (row c holds 32 copies of decode[c] then 32 of alpha[c]), so a warp's 32
// random lookups hit 32 distinct banks; the address is one PRMT.  Encode
// computes a candidate code from lg2/ex2 and corrects it with one comparison
// against the exact threshold table (also replicated per lane); the result
// equals the exact threshold count for every x in [0, 1].
#pragma once
#include "device_common.cuh"

namespace nvpyr {

constexpr uint32_t kThrRows = 255;                            // encoder candidates stay <= 254
constexpr uint32_t kLutDecodeBytes = 256 * 256;               // 256 rows x 256 B
constexpr uint32_t kLutThrBytes = kThrRows * 128;             // 255 rows x 128 B

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ float lg2Approx(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float ex2Approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Lane constants for the replicated tables (shared-window addresses).
struct Lut {
  uint32_t decBase;   // the decode table
  uint32_t laneWord;  // byte0 = 4*lane, byte1 = 4*lane + 128 (alpha half of a row)
  uint32_t thrBase;   // threshold table + 4*lane - (0x4B400000 << 7)  (see encodeChannel)
};

// decTable / thrTable: shared-window addresses of the replicated tables
// (fillLut).
__device__ __forceinline__ Lut makeLutAt(uint32_t decTable, uint32_t thrTable, uint32_t lane) {
  Lut L;
  L.decBase = decTable;
  L.laneWord = (4 * lane) | ((4 * lane + 128) << 8);
  L.thrBase = thrTable + 4 * lane - (0x4B400000u << 7);
  return L;
}

// Global-memory copy of the three tables (decode, alpha decode, encode
// thresholds), the source of fillLut: plain loads of it can all be in flight
// at once, where constant-bank loads of varying addresses are serviced one
// miss at a time.
static __device__ const uint32_t g_srgbTables[3][256] = {
    {NVPYR_SRGB_DECODE_BITS}, {NVPYR_ALPHA_DECODE_BITS}, {NVPYR_SRGB_ENCODE_THRESHOLD_BITS}};

// Fill the replicated tables: decode rows of 256 B (32 copies of decode[c],
// then 32 of alpha[c]) and threshold rows of 128 B (32 copies).  Each thread
// takes whole table entries (e = tid, tid + nthreads, ...): it loads up to
// kBatch before storing any, so with kBatch * nthreads >= 768 the whole fill
// waits for one round trip to memory, then writes each entry's 32 copies as eight 16-byte stores, lane l
// starting at 16-byte chunk l % 8 of the row so that a warp's stores spread
// over all banks (four lanes per chunk: the four wavefronts a 16-byte store
// of a warp takes anyway).
template <uint32_t kBatch = 2>
__device__ __forceinline__ void fillLut(float* dec, float* thr, uint32_t tid, uint32_t nthreads) {
  constexpr uint32_t kEntries = 3 * 256;
  const uint32_t rot = tid & 7;
  for (uint32_t e0 = tid; e0 < kEntries; e0 += kBatch * nthreads) {
    uint32_t v[kBatch];
#pragma unroll
    for (uint32_t b = 0; b < kBatch; ++b) {
      const uint32_t e = min(e0 + b * nthreads, kEntries - 1);
      v[b] = __ldg(&g_srgbTables[e >> 8][e & 255]);
    }
#pragma unroll
    for (uint32_t b = 0; b < kBatch; ++b) {
      const uint32_t e = e0 + b * nthreads, table = e >> 8, code = e & 255;
      if (e >= kEntries || (table == 2 && code >= kThrRows)) continue;
      // the entry's 32 copies: decode row c words 0..31 (table 0) or 32..63
      // (table 1), threshold row c words 0..31 (table 2)
      float4* const row = reinterpret_cast<float4*>(table == 2 ? thr + code * 32 : dec + code * 64 + table * 32);
      const float f = __uint_as_float(v[b]);
      const float4 q = make_float4(f, f, f, f);
#pragma unroll
      for (uint32_t j = 0; j < 8; ++j) row[(j + rot) & 7] = q;
    }
  }
}

__device__ __forceinline__ float lds(uint32_t addr) {
  float r;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(r) : "r"(addr));
  return r;
}

// NVPRO_PYRAMID_LOAD of one sRGBA8 texel: decode[r], decode[g], decode[b], alpha[a].
__device__ __forceinline__ float4 decodeTexel(uint32_t w, const Lut& L) {
  // PRMT builds (code << 8) | laneByte: row = code, column = this lane's copy.
  return make_float4(lds(L.decBase + __byte_perm(w, L.laneWord, 0x6604)),
                     lds(L.decBase + __byte_perm(w, L.laneWord, 0x6614)),
                     lds(L.decBase + __byte_perm(w, L.laneWord, 0x6624)),
                     lds(L.decBase + __byte_perm(w, L.laneWord, 0x6635)));
}

// Exact sRGB code of x in [0, 1], returned in the low byte.  With
//   y  = 255 * OETF(x) + 0.5   (code = floor(y)),
//   zp = 269.025 x^(5/12) - 14.925 = y - 1.4 on the power segment,
//   zl = min(3294.6 x - 0.5, 9.4)  = y - 1   on the linear segment (capped),
// z = max(zp, zl) lies in [y - 1.4, y - 1] up to ~1e-3, so a = rn(z) is code-1
// or code, and code = a + (x >= threshold[a]).  z >= -0.5 (rounds to 0) and
// z <= 254.1, so a indexes rows 0..254.  The magic add leaves a in the low
// bits of `bits`, and (bits << 7) + thrBase is the address of threshold[a].
__device__ __forceinline__ uint32_t encodeChannel(float x, const Lut& L) {
  const float p = ex2Approx(lg2Approx(x) * 0.41666666f);
  const float zp = fmaf(p, 269.025f, -14.925f);
  const float zl = fminf(fmaf(x, 3294.6f, -0.5f), 9.4f);
  const uint32_t bits = __float_as_uint(fmaxf(zp, zl) + 12582912.0f);
  const float thr = lds(bits * 128u + L.thrBase);
  return bits + (x >= thr ? 1u : 0u);
}

// srgbFromLinearVec's alpha: uint(a * 255 + 0.5) with truncation, via a
// round-toward-zero add that leaves the integer in the low mantissa bits.
__device__ __forceinline__ uint32_t encodeAlpha(float a) {
  const float s = __fadd_rn(__fmul_rn(a, 255.0f), 0.5f);
  return __float_as_uint(__fadd_rz(s, 8388608.0f));
}

// encodeChannel x3 + encodeAlpha with the independent multiplies and adds of
// the colour channels paired into packed FP32 instructions.  The colour codes
// only need a candidate within one of the true code (the threshold compare
// corrects it), so their arithmetic may round or fuse freely.  Alpha is exact
// arithmetic, uint(rn(rn(a * 255) + 0.5)): it uses __fmul_rn / __fadd_rn,
// which are never merged into a multiply-add.
__device__ __forceinline__ uint32_t encodeTexel(float4 v, const Lut& L) {
  constexpr float k = 0.41666666f, magic = 12582912.0f;
  const float2 tRG = __fmul2_rn(make_float2(lg2Approx(v.x), lg2Approx(v.y)), make_float2(k, k));
  const float tB = lg2Approx(v.z) * k;
  const float s = __fadd_rn(__fmul_rn(v.w, 255.0f), 0.5f);
  const float2 pRG = make_float2(ex2Approx(tRG.x), ex2Approx(tRG.y));
  const float pB = ex2Approx(tB);
  const float2 zpRG = __ffma2_rn(pRG, make_float2(269.025f, 269.025f), make_float2(-14.925f, -14.925f));
  const float zpB = fmaf(pB, 269.025f, -14.925f);
  const float2 zlRG = __ffma2_rn(make_float2(v.x, v.y), make_float2(3294.6f, 3294.6f), make_float2(-0.5f, -0.5f));
  const float zlB = fmaf(v.z, 3294.6f, -0.5f);
  const float2 mRG = __fadd2_rn(make_float2(fmaxf(zpRG.x, fminf(zlRG.x, 9.4f)), fmaxf(zpRG.y, fminf(zlRG.y, 9.4f))),
                                make_float2(magic, magic));
  const uint32_t bR = __float_as_uint(mRG.x), bG = __float_as_uint(mRG.y);
  const uint32_t bB = __float_as_uint(fmaxf(zpB, fminf(zlB, 9.4f)) + magic);
  const uint32_t r = bR + (v.x >= lds(bR * 128u + L.thrBase) ? 1u : 0u);
  const uint32_t g = bG + (v.y >= lds(bG * 128u + L.thrBase) ? 1u : 0u);
  const uint32_t b = bB + (v.z >= lds(bB * 128u + L.thrBase) ? 1u : 0u);
  const uint32_t a = __float_as_uint(__fadd_rz(s, 8388608.0f));
  return __byte_perm(__byte_perm(r, g, 0x0040), __byte_perm(b, a, 0x0040), 0x5410);
}

// The value a dispatch hands on to its next level through the reference's
// shared memory, in the pipeline's shared format SF
// (srgba8_mipmap_preamble.glsl:60-108): FP32 unchanged; SRGB_SHARED the
// texel's sRGBA8 code decoded again; F16_SHARED each channel as binary16.
template <uint32_t SF>
__device__ __forceinline__ float4 sharedRoundTrip(float4 v, const Lut& L) {
  if (SF == kSharedSrgb) return decodeTexel(encodeTexel(v, L), L);
  if (SF == kSharedF16) return f16RoundTrip(v);
  return v;
}

// REDUCE4 on packed pairs: 0.25 * ((v00 + v01) + (v10 + v11)) per channel,
// same operations and order as reduce4().
__device__ __forceinline__ float4 add4p(float4 a, float4 b) {
  const float2 lo = __fadd2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y));
  const float2 hi = __fadd2_rn(make_float2(a.z, a.w), make_float2(b.z, b.w));
  return make_float4(lo.x, lo.y, hi.x, hi.y);
}
__device__ __forceinline__ float4 reduce4p(float4 v00, float4 v01, float4 v10, float4 v11) {
  const float4 t = add4p(add4p(v00, v01), add4p(v10, v11));
  const float2 lo = __fmul2_rn(make_float2(0.25f, 0.25f), make_float2(t.x, t.y));
  const float2 hi = __fmul2_rn(make_float2(0.25f, 0.25f), make_float2(t.z, t.w));
  return make_float4(lo.x, lo.y, hi.x, hi.y);
}
__device__ __forceinline__ float4 fastReduceP(bool vertical, float4 tl, float4 tr, float4 bl, float4 br) {
  return vertical ? reduce4p(tl, bl, tr, br) : reduce4p(tl, tr, bl, br);
}

__device__ __forceinline__ float4 shflXor(float4 v, int m) {
  return make_float4(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m),
                     __shfl_xor_sync(0xffffffffu, v.z, m), __shfl_xor_sync(0xffffffffu, v.w, m));
}
__device__ __forceinline__ float4 shflDown(float4 v, int d) {
  return make_float4(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d),
                     __shfl_down_sync(0xffffffffu, v.z, d), __shfl_down_sync(0xffffffffu, v.w, d));
}
__device__ __forceinline__ float4 shflUp(float4 v, int d) {
  return make_float4(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d),
                     __shfl_up_sync(0xffffffffu, v.z, d), __shfl_up_sync(0xffffffffu, v.w, d));
}

}  // namespace nvpyr
