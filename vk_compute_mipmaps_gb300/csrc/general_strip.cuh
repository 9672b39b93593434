// general_strip.cuh -- the column-strip machinery of the sRGBA8 general
// pipeline (nvpro_pyramid.glsl:536-885), shared by the chain kernel
// (kernels_general.cu) and the batch kernel (kernels_batch.cu): the strip
// walk, its FP32 arithmetic in the reference's operation order, the aligned
// sRGB decode, and the bounded grid barrier between dispatches.
//
// A strip is one warp's unit of work: a band of rows of the last level of
// the dispatch, 31 columns of level L+2 (two levels) or 63 columns of level
// L+1 (one level).  Lane l owns two level-(L+1) columns and loads the four
// level-L columns under them; a three-tap window's third column is lane
// l+1's first (shfl.down 1).  The warp walks the band top to bottom, two
// level-(L+1) rows per step: it reduces the new level-L rows vertically per
// column, then horizontally (vertical first, as reduceStoreSample_ does,
// :588-651), stores the encoded texels, and keeps the FP32 values for level
// L+2, which reduces the same way over the lanes' level-(L+1) values
// (fillLastTile_ reads FP32 level L+1 from shared memory, :790-820; here it
// comes from registers).  The level-L rows of the next step are in flight
// while the current one is reduced.
//
// Every texel's value depends only on its inputs and the fixed operation
// order, so strips overlap by one level-(L+1) column / row where a three-tap
// window crosses a strip edge; the overlapping texels are recomputed and
// stored by one strip only.  The results equal the portable kernels' bytes.
#pragma once
#include "srgb_codec.cuh"

namespace nvpyr {
namespace {

constexpr uint32_t kCols2 = 31;     // level-(L+2) columns per strip (two levels)
constexpr uint32_t kCols1 = 63;     // level-(L+1) columns per strip (one level)
constexpr uint32_t kWaitLimit = 1u << 22;  // grid barrier polls (with backoff: about a second)
constexpr uint32_t kTightPolls = 512;      // polls before the backoff starts

// The replicated sRGB tables with the decode table at a 64 KiB boundary of
// the shared window (decodeAligned): the threshold table below it if it fits
// there, else above it; 128 KiB of dynamic shared memory cover every placement.
constexpr uint32_t kAlignedLutSmemBytes = 2 * kLutDecodeBytes;
// One dispatch (a stage of a chain launch).
struct Stage {
  const uint8_t* src;
  uint64_t srcPitch;
  uint32_t w0, h0;
  uint8_t* dst1;
  uint64_t pitch1;
  uint32_t w1, h1;
  uint8_t* dst2;
  uint64_t pitch2;
  uint32_t w2, h2;
  uint32_t tilesX;   // strips across the last level
  uint32_t bands;    // bands down the last level
  uint32_t band;     // rows of the last level per band
  uint32_t variant;  // two levels: tx0<<3 | ty0<<2 | tx1<<1 | ty1; one level: 16 + (tx0<<1 | ty0)
};

// REDUCE / REDUCE2 (srgba8_mipmap_preamble.glsl:24-38), equal to reduce3() /
// reduce2(): products on packed pairs (__fmul2_rn).  The sums of REDUCE stay
// scalar (__fadd_rn): with packed adds (__fadd2_rn) after the packed products
// one alpha byte of a 255x256 chain came out one off, also when compiled with
// -fmad=false.  REDUCE2's add may be
// packed: its operands are decoded values, sums, or exact halvings
// (0.5 * x), and the parity tests hold for it.
__device__ __forceinline__ float4 mul4p(float s, float4 a) {
  const float2 lo = __fmul2_rn(make_float2(s, s), make_float2(a.x, a.y));
  const float2 hi = __fmul2_rn(make_float2(s, s), make_float2(a.z, a.w));
  return make_float4(lo.x, lo.y, hi.x, hi.y);
}
__device__ __forceinline__ float4 reduce3p(const Weights3& w, float4 v0, float4 v1, float4 v2) {
  return f4add(f4add(mul4p(w.w0, v0), mul4p(w.w1, v1)), mul4p(w.w2, v2));
}
__device__ __forceinline__ float4 reduce2p(float4 v0, float4 v1) { return mul4p(0.5f, add4p(v0, v1)); }

// weights3(n, i) with the reciprocal 1 / (2n + 1) computed once per level.
struct Axis3 {
  float nf, rcp;
};
__device__ __forceinline__ Axis3 axis3(uint32_t n) {
  const float nf = __uint2float_rn(n);
  return Axis3{nf, __frcp_rn(__fadd_rn(__fmul_rn(2.0f, nf), 1.0f))};
}
__device__ __forceinline__ Weights3 weightsAt(const Axis3& a, uint32_t i) {
  Weights3 w;
  w.w0 = __fmul_rn(a.rcp, __fsub_rn(a.nf, __uint2float_rn(i)));
  w.w1 = __fmul_rn(a.rcp, a.nf);
  w.w2 = __fsub_rn(__fsub_rn(1.0f, w.w0), w.w1);
  return w;
}

// L2-coherent texel load (ld.global.cg): the level may have been written by
// another SM earlier in the same launch, and a 32-byte sector at the end of
// one level can hold the first bytes of the next, so no L1 copy is trusted.
// Volatile keeps the prefetch ahead of the table lookups.
__device__ __forceinline__ uint32_t ldTexel(const uint8_t* p) {
  uint32_t v;
  asm volatile("ld.global.cg.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}

// Steps of level-L rows a strip asks L2 for beyond the rows it holds in
// registers (prefetch.global.L2: no registers, no completion): the loads of
// those rows, one step ahead of their use, then hit L2.
constexpr uint32_t kStripL2Steps = 2;

__device__ __forceinline__ void prefetchL2(const uint8_t* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Store `v` to `p` if `pred`: a predicated st.global, so the value (an
// encode every lane computes anyway) is not moved into a divergent branch.
__device__ __forceinline__ void storeIf(bool pred, uint8_t* p, uint32_t v) {
  asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n @q st.global.u32 [%0], %1;\n}\n" ::"l"(p), "r"(v),
               "r"(uint32_t(pred))
               : "memory");
}

// decodeTexel for a decode table at a 64 KiB-aligned shared address: the
// PRMT builds the whole address, table bytes 2-3 coming from laneWord.
__device__ __forceinline__ float4 decodeAligned(uint32_t w, const Lut& L) {
  return make_float4(lds(__byte_perm(w, L.laneWord, 0x7604)), lds(__byte_perm(w, L.laneWord, 0x7614)),
                     lds(__byte_perm(w, L.laneWord, 0x7624)), lds(__byte_perm(w, L.laneWord, 0x7635)));
}

// One strip of a one- or two-level dispatch.  TX0 / TY0: three-tap kernel
// from level L along x / y (else two taps); TX1 / TY1: the same from level
// L+1 (two levels only).  The flags are read once from the stage's variant;
// they are uniform across the grid, so their branches never diverge.  SF: the
// pipeline's shared format, applied to the level-(L+1) values that level L+2
// is reduced from (sharedLevel_, nvpro_pyramid.glsl:664,717).
//
// Lane l owns level-(L+1) columns xa = x0 + 2l and xb = xa + 1 and level-(L+2)
// column X0 + l, and loads level-L columns 2xa .. 2xa + 3; the third tap
// 2xb + 2 of xb is lane l+1's first column, and the third level-(L+1) column
// 2X + 2 of X is lane l+1's xa (shfl.down 1 of the vertically reduced values).
// A strip is 31 level-(L+2) columns (62 level-(L+1) columns stored; lane 31
// only feeds lane 30, and stores xa in the last strip) or 63 level-(L+1)
// columns for one-level dispatches.  Each step reduces two level-(L+1) rows
// (rA, rB = rA + 1) from four new level-L rows and, for two levels, one
// level-(L+2) row; the next step's four rows load while this one reduces.
// Operation order (reduceStoreSample_, nvpro_pyramid.glsl:575-656): per
// column vertical first, then horizontal, every multiply and add rounded
// separately, as in the oracle.
__device__ __forceinline__ float4 colReduce(bool three, const Weights3& w, float4 a, float4 b, float4 c) {
  return three ? reduce3p(w, a, b, c) : reduce2p(a, b);
}

template <uint32_t SF>
__device__ __forceinline__ void strip(const Stage& st, uint32_t tile, uint32_t band, uint32_t lane, const Lut& lut) {
  const uint32_t variant = st.variant;
  const bool two = variant < 16;
  const bool TX0 = two ? (variant & 8) != 0 : (variant & 2) != 0;
  const bool TY0 = two ? (variant & 4) != 0 : (variant & 1) != 0;
  const bool TX1 = two && (variant & 2) != 0;
  const bool TY1 = two && (variant & 1) != 0;
  // Every field in a register before the first store: stores through
  // generic pointers would otherwise force reloads of a stage held in memory.
  const Lut L = lut;
  const uint8_t* const src = st.src;
  const uint64_t pitch = st.srcPitch;
  const uint32_t w0 = st.w0;
  uint8_t* const dst1 = st.dst1;
  const uint64_t pitch1 = st.pitch1;
  const uint32_t w1 = st.w1, h1 = st.h1;
  uint8_t* const dst2 = st.dst2;
  const uint64_t pitch2 = st.pitch2;
  const uint32_t w2 = st.w2, h2 = st.h2, bandRows = st.band;

  const uint32_t x0 = tile * (two ? 2 * kCols2 : kCols1);
  const uint32_t xa = x0 + 2 * lane, xb = xa + 1;
  const bool lastTile = (tile + 1) * (two ? kCols2 : kCols1) >= (two ? w2 : w1);
  // lane 31's xa belongs to a one-level strip (63 columns); in a two-level one
  // it is the next strip's first column, except in the last strip
  const bool storeA = xa < w1 && (lane < 31 || !two || lastTile);
  const bool storeB = xb < w1 && lane < 31;
  const uint32_t X = x0 / 2 + lane;  // this lane's level-(L+2) column
  const bool storeX = two && lane < 31 && X < w2;
  // level-L columns 2xa .. 2xa + 3, clamped into the level (clamped ones feed
  // no stored texel)
  const uint32_t ca = min(2 * xa, w0 - 1);
  const uint8_t* const colA = src + uint64_t(ca) * 4;
  const uint32_t d1 = (min(2 * xa + 1, w0 - 1) - ca) * 4, d2 = (min(2 * xa + 2, w0 - 1) - ca) * 4,
                 d3 = (min(2 * xa + 3, w0 - 1) - ca) * 4;
  const Axis3 ax1 = axis3(w1), ay1 = axis3(h1), ax2 = axis3(w2), ay2 = axis3(h2);
  const Weights3 wxa = weightsAt(ax1, min(xa, w1 - 1)), wxb = weightsAt(ax1, min(xb, w1 - 1));
  const Weights3 wX = weightsAt(ax2, min(X, w2 - 1));

  // level-(L+1) rows [yb, ye) of this band, of which [yb, yStoreEnd) are stored here
  uint32_t yb, ye, yStoreEnd;
  if (two) {
    const uint32_t Yb = band * bandRows, Ye = min(Yb + bandRows, h2);
    yb = 2 * Yb;
    ye = 2 * Ye + (TY1 ? 1 : 0);
    yStoreEnd = Ye == h2 ? h1 : 2 * Ye;
  } else {
    yb = band * bandRows;
    ye = min(yb + bandRows, h1);
    yStoreEnd = ye;
  }

  // four level-L rows from `row0`, the lane's four columns each; rows at or
  // beyond `rowEnd` are not read
  auto ldRows = [&](uint32_t row0, uint32_t rowEnd, uint32_t (&raw)[4][4]) {
    const uint8_t* p = colA + uint64_t(row0) * pitch;
#pragma unroll
    for (uint32_t j = 0; j < 4; ++j) {
      if (row0 + j < rowEnd) {
        raw[j][0] = ldTexel(p);
        raw[j][1] = ldTexel(p + d1);
        raw[j][2] = ldTexel(p + d2);
        raw[j][3] = ldTexel(p + d3);
      }
      p += pitch;
    }
  };
  // ask L2 for four level-L rows from `row0` (one address per lane: the
  // lanes' 16-byte column groups cover the strip's span of the row)
  auto pfRows = [&](uint32_t row0, uint32_t rowEnd) {
    const uint8_t* p = colA + uint64_t(row0) * pitch;
#pragma unroll
    for (uint32_t j = 0; j < 4; ++j) {
      if (row0 + j < rowEnd) prefetchL2(p);
      p += pitch;
    }
  };
  auto decodeRow = [&](const uint32_t (&r)[4], float4 (&d)[4]) {
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) d[k] = decodeAligned(r[k], L);
  };

  // Level-(L+1) row y from level-L rows (carry = row 2y when TY0, r1, r2):
  // vertical per column, then the two horizontal reductions; stores them and
  // returns their FP32 values (after the shared format) in a / b.
  float4 carry[4];  // TY0: decoded level-L row 2y of the next level-(L+1) row
  auto level1Row = [&](uint32_t y, const uint32_t (&r1)[4], const uint32_t (&r2)[4], float4& a, float4& b) {
    float4 d1v[4], d2v[4], v[4];
    decodeRow(r1, d1v);
    decodeRow(r2, d2v);
    if (TY0) {
      const Weights3 wy = weightsAt(ay1, y);
#pragma unroll
      for (uint32_t k = 0; k < 4; ++k) v[k] = reduce3p(wy, carry[k], d1v[k], d2v[k]);
#pragma unroll
      for (uint32_t k = 0; k < 4; ++k) carry[k] = d2v[k];
    } else {
#pragma unroll
      for (uint32_t k = 0; k < 4; ++k) v[k] = reduce2p(d1v[k], d2v[k]);
    }
    const float4 v4 = shflDown(v[0], 1);
    a = colReduce(TX0, wxa, v[0], v[1], v[2]);
    b = TX0 ? reduce3p(wxb, v[2], v[3], v4) : reduce2p(v[2], v[3]);
    const uint32_t ea = encodeTexel(a, L), eb = encodeTexel(b, L);
    const bool rowOk = y < yStoreEnd;
    uint8_t* const out = dst1 + uint64_t(y) * pitch1 + uint64_t(xa) * 4;
    storeIf(storeA && rowOk, out, ea);
    storeIf(storeB && rowOk, out + 4, eb);
    if (SF == kSharedSrgb) {
      a = decodeAligned(ea, L);
      b = decodeAligned(eb, L);
    }
    if (SF == kSharedF16) {
      a = f16RoundTrip(a);
      b = f16RoundTrip(b);
    }
  };

  // first level-(L+1) row of the steps: rA = yb (+1 when TY1: row yb comes first, alone)
  const uint32_t l0End = 2 * ye + (TY0 ? 1 : 0);  // level-L rows this band reads: [.., l0End)
  float4 pa = make_float4(0.f, 0.f, 0.f, 0.f), pb = pa;  // TY1: level-(L+1) row 2Y of the next level-(L+2) row
  // The band's first level-L rows are all requested before any is used: the
  // carry row (TY0), the two rows of the lone level-(L+1) row (TY1) and the
  // four rows of the first step, so a short band waits for one round trip
  // to memory, not three.
  const uint32_t off = TY0 ? 1 : 0;
  uint32_t y = yb + (TY1 ? 1 : 0);  // the first step's level-(L+1) row
  uint32_t r0[4], rT[4][4], bufA[4][4], bufB[4][4];
  if (TY0) {  // level-L row 2yb
    const uint8_t* p = colA + uint64_t(2 * yb) * pitch;
    r0[0] = ldTexel(p);
    r0[1] = ldTexel(p + d1);
    r0[2] = ldTexel(p + d2);
    r0[3] = ldTexel(p + d3);
  }
  if (TY1) ldRows(2 * yb + off, 2 * yb + off + 2, rT);  // level-L rows of level-(L+1) row yb
  if (y < ye) ldRows(2 * y + off, l0End, bufA);
  if (TY0) decodeRow(r0, carry);
  if (TY1) level1Row(yb, rT[0], rT[1], pa, pb);  // the top row of the first level-(L+2) row
  // steps of two level-(L+1) rows (y, y + 1); level-L rows from 2y (+1 with TY0)
#pragma unroll
  for (uint32_t k = 2; k <= kStripL2Steps; ++k)  // the steps before the loop's first prefetch
    if (y + 2 * k < ye) pfRows(2 * (y + 2 * k) + off, l0End);
  auto step = [&](uint32_t yy, const uint32_t (&r)[4][4]) {
    float4 aA, bA, aB = make_float4(0.f, 0.f, 0.f, 0.f), bB = aB;
    level1Row(yy, r[0], r[1], aA, bA);
    if (yy + 1 < ye) level1Row(yy + 1, r[2], r[3], aB, bB);
    if (two) {
      // level-(L+2) row Y from level-(L+1) rows 2Y (pa, pb), 2Y+1, 2Y+2 (TY1) or 2Y, 2Y+1
      float4 ua, ub;
      uint32_t Y;
      if (TY1) {
        Y = (yy - 1) >> 1;
        const Weights3 wY = weightsAt(ay2, Y);
        ua = reduce3p(wY, pa, aA, aB);
        ub = reduce3p(wY, pb, bA, bB);
        pa = aB;
        pb = bB;
      } else {
        Y = yy >> 1;
        ua = reduce2p(aA, aB);
        ub = reduce2p(bA, bB);
      }
      const float4 uc = shflDown(ua, 1);
      const float4 o = TX1 ? reduce3p(wX, ua, ub, uc) : reduce2p(ua, ub);
      storeIf(storeX, dst2 + uint64_t(Y) * pitch2 + uint64_t(X) * 4, encodeTexel(o, L));
    }
  };
  constexpr uint32_t kPfRows = 2 * (kStripL2Steps + 1);  // level-(L+1) rows ahead of y
  for (;;) {
    if (y >= ye) break;
    if (y + 2 < ye) ldRows(2 * (y + 2) + off, l0End, bufB);
    if (kStripL2Steps && y + kPfRows < ye) pfRows(2 * (y + kPfRows) + off, l0End);
    step(y, bufA);
    y += 2;
    if (y >= ye) break;
    if (y + 2 < ye) ldRows(2 * (y + 2) + off, l0End, bufA);
    if (kStripL2Steps && y + kPfRows < ye) pfRows(2 * (y + kPfRows) + off, l0End);
    step(y, bufB);
    y += 2;
  }
}

__device__ __forceinline__ uint32_t ldAcquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier between stages (all CTAs are resident: cooperative launch).
// Thread 0 of each CTA arrives on the counter after a release fence; the last
// arrival resets the counter and publishes generation `gen + 1`; the others
// poll the generation with nanosleep backoff, at most kWaitLimit times.
// Returns false (after setting the error flag) if the wait gave up.
__device__ __forceinline__ bool gridBarrierWait(uint32_t* count, uint32_t* genWord, uint32_t* errorFlag, uint32_t& gen,
                                                uint32_t* okFlag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t ok = 1;
    const uint32_t next = gen + 1;
    __threadfence();
    if (atomicAdd(count, 1u) == gridDim.x - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicExch(genWord, next);
    } else {
      // a short tight spin (the last CTAs of a stage arrive close together),
      // then polls with backoff
      uint32_t it = 0;
      while (ldAcquire(genWord) != next) {
        if (++it >= kWaitLimit) {
          atomicExch(errorFlag, 1u);
          ok = 0;
          break;
        }
        if (it > kTightPolls) __nanosleep(256);
      }
    }
    __threadfence();
    *okFlag = ok;
  }
  __syncthreads();
  ++gen;
  return *okFlag != 0;
}

// Host side: a stage's level views, kernel variant and strips across the
// last level (everything but the band height).
inline void stageGeometry(const DispatchParams& p, Stage* g) {
  *g = Stage{};
  g->src = p.lv[0].ptr;
  g->srcPitch = p.lv[0].pitch;
  g->w0 = p.lv[0].w;
  g->h0 = p.lv[0].h;
  g->dst1 = p.lv[1].ptr;
  g->pitch1 = p.lv[1].pitch;
  g->w1 = p.lv[1].w;
  g->h1 = p.lv[1].h;
  const bool two = p.levelCount == 2;
  if (two) {
    g->dst2 = p.lv[2].ptr;
    g->pitch2 = p.lv[2].pitch;
    g->w2 = p.lv[2].w;
    g->h2 = p.lv[2].h;
  } else {
    g->w2 = g->h2 = 1;
  }
  const bool tx0 = kernelSize(g->w0) == 3, ty0 = kernelSize(g->h0) == 3;
  const bool tx1 = two && kernelSize(g->w1) == 3, ty1 = two && kernelSize(g->h1) == 3;
  g->variant = two ? ((tx0 ? 8u : 0u) | (ty0 ? 4u : 0u) | (tx1 ? 2u : 0u) | (ty1 ? 1u : 0u))
                   : 16u + (tx0 ? 2u : 0u) + (ty0 ? 1u : 0u);
  const uint32_t lastW = two ? g->w2 : g->w1;
  g->tilesX = (lastW + (two ? kCols2 : kCols1) - 1) / (two ? kCols2 : kCols1);
}

// Band height (rows of the last level, at least 1) and band count.
inline void setStageBand(Stage* g, uint32_t band) {
  const uint32_t lastH = g->variant < 16 ? g->h2 : g->h1;
  band = band < 1 ? 1 : (band > lastH ? lastH : band);
  g->band = band;
  g->bands = (lastH + band - 1) / band;
}

// The last CTA to arrive returns true (the others false and may exit): a
// hand-off without waiting.  Writes of every CTA before its arrival are
// visible to the last one after (release / acquire fences around the count).
__device__ __forceinline__ bool lastCtaArrives(uint32_t* count, uint32_t* flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const bool last = atomicAdd(count, 1u) == gridDim.x - 1;
    if (last) {
      atomicExch(count, 0u);
      __threadfence();
    }
    *flag = last ? 1u : 0u;
  }
  __syncthreads();
  return *flag != 0;
}

// The sRGB codec through the tables of fillAlignedLut: the decode table's
// address comes whole from the PRMT (decodeAligned), since the Lut's lane word
// carries the table's upper address bytes.
struct AlignedLutCodec {
  Lut L;
  __device__ __forceinline__ float4 decode(uint32_t w) const { return decodeAligned(w, L); }
  __device__ __forceinline__ uint32_t encode(float4 v) const { return encodeTexel(v, L); }
};

// Fill the aligned tables in `smem` (kAlignedLutSmemBytes of dynamic shared
// memory) and return the lane's table constants.  Call with every thread of
// the CTA; a __syncthreads must follow before the first lookup.
template <uint32_t kBatch = 2>
__device__ __forceinline__ Lut fillAlignedLut(uint8_t* smem, uint32_t tid, uint32_t nthreads) {
  const uint32_t base = smemAddr(smem);
  const uint32_t decOff = (0x10000u - (base & 0xFFFFu)) & 0xFFFFu;
  const uint32_t thrOff = decOff >= kLutThrBytes ? 0u : decOff + kLutDecodeBytes;
  fillLut<kBatch>(reinterpret_cast<float*>(smem + decOff), reinterpret_cast<float*>(smem + thrOff), tid, nthreads);
  Lut L = makeLutAt(base + decOff, base + thrOff, tid & 31);
  L.laneWord |= (base + decOff) & 0xFFFF0000u;  // table bytes 2-3 for decodeAligned
  return L;
}

}  // namespace
}  // namespace nvpyr
