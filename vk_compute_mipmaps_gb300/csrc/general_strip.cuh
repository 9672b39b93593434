// general_strip.cuh -- the column-strip machinery of the sRGBA8 general
// pipeline (nvpro_pyramid.glsl:536-885), shared by the chain kernel
// (kernels_general.cu) and the batch kernel (kernels_batch.cu): the strip
// walk, its FP32 arithmetic in the reference's operation order, the aligned
// sRGB decode, and the bounded grid barrier between dispatches.
//
// A strip is one warp's unit of work: a band of rows of the last level of
// the dispatch, 15 columns of level L+2 (two levels) or 31 columns of level
// L+1 (one level).  Lane l owns level-(L+1) column x = x0 + l and loads
// level-L columns 2x and 2x+1; a three-tap column 2x+2 is lane l+1's first
// column (shfl.down 1).  The warp walks the band's level-(L+1) rows top to
// bottom: each row reads two new level-L rows (the third row of a three-tap
// window is the previous row's last), reduces them vertically per column,
// then horizontally across lanes (vertical first, as reduceStoreSample_
// does, :588-651), stores the encoded texel, and keeps the FP32 value for
// level L+2, which reduces the same way over the lanes' level-(L+1) rows
// (fillLastTile_ reads FP32 level L+1 from shared memory, :790-820; here it
// comes from registers).  The level-L rows of the next four level-(L+1) rows
// are in flight while the current four are reduced.
//
// Every texel's value depends only on its inputs and the fixed operation
// order, so strips overlap by one level-(L+1) column / row where a three-tap
// window crosses a strip edge; the overlapping texels are recomputed and
// stored by one strip only.  The results equal the portable kernels' bytes.
#pragma once
#include "srgb_codec.cuh"

namespace nvpyr {
namespace {

constexpr uint32_t kCols2 = 15;     // level-(L+2) columns per strip (two levels)
constexpr uint32_t kCols1 = 31;     // level-(L+1) columns per strip (one level)
constexpr uint32_t kGroupRows = 4;  // level-(L+1) rows whose level-L rows load together
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
// reduce2(): products on packed pairs (__fmul2_rn).  The sums of REDUCE must
// stay scalar: __fadd_rn is never merged into a multiply-add, while packed
// adds next to packed multiplies were seen fused (a fused w0*v0 + w1*v1
// changes encoded bytes).  REDUCE2's add may be packed: its operands are
// decoded values, sums, or exact halvings (0.5 * x), so a fused and an
// unfused result are the same.
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
// L+1 (two levels only).  The flags are uniform across the grid, so their
// branches never diverge; one code path for all of them keeps the chain
// kernel free of calls.  SF: the pipeline's shared format, applied to the
// level-(L+1) values that level L+2 is reduced from (sharedLevel_,
// nvpro_pyramid.glsl:664,717).
// strip<SF, V>: V fixes the stage's variant at compile time, or kRuntimeVariant
// reads it once from the stage (measured: a single read of the variant instead
// of one per flag took 4095^2 from 75.8 to 73.7 us and the 256-image batch
// from 1454 to 1375 us; a second, variant-15 copy in the chain kernel spilled).
constexpr uint32_t kRuntimeVariant = 255;

// ROWS: level-(L+1) rows whose level-L rows load together (the prefetch
// depth); 4 in the chain kernel, 2 in the batch kernel, whose units are
// shorter (measured: 2 rows took the 256-image batch from 1375 to 1313 us
// but the 4095^2 chain from 74 to 78 us).
template <uint32_t SF, uint32_t V = kRuntimeVariant, uint32_t ROWS = kGroupRows>
__device__ __forceinline__ void strip(const Stage& st, uint32_t tile, uint32_t band, uint32_t lane, const Lut& lut) {
  const uint32_t variant = V == kRuntimeVariant ? st.variant : V;
  const uint32_t LEVELS = variant >= 16 ? 1u : 2u;
  const bool TX0 = LEVELS == 2 ? (variant & 8) != 0 : (variant & 2) != 0;
  const bool TY0 = LEVELS == 2 ? (variant & 4) != 0 : (variant & 1) != 0;
  const bool TX1 = LEVELS == 2 && (variant & 2) != 0;
  const bool TY1 = LEVELS == 2 && (variant & 1) != 0;
  // Every field in a register before the first store: stores through
  // generic pointers would otherwise force reloads of a stage held in memory.
  const Lut L = lut;
  struct {
    const uint8_t* src;
    uint64_t srcPitch;
    uint32_t w0, h0;
    uint8_t* dst1;
    uint64_t pitch1;
    uint32_t w1, h1;
    uint8_t* dst2;
    uint64_t pitch2;
    uint32_t w2, h2, band;
  } const p = {st.src, st.srcPitch, st.w0, st.h0, st.dst1, st.pitch1, st.w1, st.h1, st.dst2, st.pitch2, st.w2, st.h2,
               st.band};
  const uint32_t cols = LEVELS == 2 ? 2 * kCols2 : kCols1;  // level-(L+1) columns owned by a strip
  const uint32_t x0 = tile * cols;
  const uint32_t x = x0 + lane;
  // level-L columns of this lane, clamped into the level for lanes past its edge
  const uint8_t* colA = p.src + uint64_t(min(2 * x, p.w0 - 1)) * 4;
  const uint8_t* colB = p.src + uint64_t(min(2 * x + 1, p.w0 - 1)) * 4;
  const Axis3 ax1 = axis3(p.w1), ay1 = axis3(p.h1);
  const Weights3 wx = weightsAt(ax1, min(x, p.w1 - 1));

  // rows [yb, ye) of level L+1, of which [yb, yStoreEnd) are this strip's
  uint32_t yb, ye, yStoreEnd;
  bool store1x;
  if (LEVELS == 2) {
    const uint32_t Yb = band * p.band, Ye = min(Yb + p.band, p.h2);
    yb = 2 * Yb;
    ye = 2 * Ye + (TY1 ? 1 : 0);
    yStoreEnd = Ye == p.h2 ? p.h1 : 2 * Ye;
    const bool lastTile = (tile + 1) * kCols2 >= p.w2;
    store1x = x < p.w1 && (lane < cols || lastTile);
  } else {
    yb = band * p.band;
    ye = min(yb + p.band, p.h1);
    yStoreEnd = ye;
    store1x = x < p.w1 && lane < cols;
  }
  const uint32_t X = x0 / 2 + (lane >> 1);  // level-(L+2) column of an even lane
  const bool store2x = LEVELS == 2 && (lane & 1) == 0 && lane < 2 * kCols2 && X < p.w2;
  const Axis3 ax2 = axis3(p.w2), ay2 = axis3(p.h2);
  const Weights3 wX = weightsAt(ax2, min(X, p.w2 - 1));

  // Level-L rows: lane texels at colA / colA + dB of row r.  Rows are read
  // only while their level-(L+1) row is inside the band, so no row index
  // leaves the level (for y < ye: 2y + 2 <= h0 - 1 with three taps, 2y + 1
  // <= h0 - 1 with two).
  const uint32_t dB = uint32_t(colB - colA);  // 4, or 0 where column 2x+1 is clamped
  const uint64_t pitch = p.srcPitch;
  auto ldGroup = [&](uint32_t yg, uint32_t (&raw)[ROWS][4]) {
    const uint8_t* row = colA + uint64_t(TY0 ? 2 * yg + 1 : 2 * yg) * pitch;
#pragma unroll
    for (uint32_t j = 0; j < ROWS; ++j) {
      if (yg + j < ye) {
        raw[j][0] = ldTexel(row);
        raw[j][1] = ldTexel(row + dB);
        raw[j][2] = ldTexel(row + pitch);
        raw[j][3] = ldTexel(row + pitch + dB);
      }
      row += 2 * pitch;
    }
  };

  float4 pa = make_float4(0.f, 0.f, 0.f, 0.f), pb = pa;  // three taps: level-L row 2y
  if (TY0) {
    const uint8_t* row = colA + uint64_t(2 * yb) * pitch;
    pa = decodeAligned(ldTexel(row), L);
    pb = decodeAligned(ldTexel(row + dB), L);
  }
  float4 h0v = make_float4(0.f, 0.f, 0.f, 0.f), h1v = h0v;  // level-(L+1) rows 2Y, 2Y+1

  auto process = [&](uint32_t yg, const uint32_t (&raw)[ROWS][4]) {
#pragma unroll
    for (uint32_t j = 0; j < ROWS; ++j) {
      const uint32_t y = yg + j;
      if (y >= ye) break;
      const float4 r1a = decodeAligned(raw[j][0], L), r1b = decodeAligned(raw[j][1], L);
      const float4 r2a = decodeAligned(raw[j][2], L), r2b = decodeAligned(raw[j][3], L);
      float4 va, vb;
      if (TY0) {
        const Weights3 wy = weightsAt(ay1, y);
        va = reduce3p(wy, pa, r1a, r2a);
        vb = reduce3p(wy, pb, r1b, r2b);
        pa = r2a;
        pb = r2b;
      } else {
        va = reduce2p(r1a, r2a);
        vb = reduce2p(r1b, r2b);
      }
      float4 l1;
      if (TX0)
        l1 = reduce3p(wx, va, vb, shflDown(va, 1));
      else
        l1 = reduce2p(va, vb);
      const uint32_t code1 = encodeTexel(l1, L);
      storeIf(store1x && y < yStoreEnd, p.dst1 + uint64_t(y) * p.pitch1 + uint64_t(x) * 4, code1);
      if (LEVELS == 2) {
        if (SF == kSharedSrgb) l1 = decodeAligned(code1, L);
        if (SF == kSharedF16) l1 = f16RoundTrip(l1);
        const uint32_t jj = y - yb;
        bool emit = false;
        uint32_t Y = 0;
        float4 v2 = l1;
        if (TY1) {
          if (jj == 0) {
            h0v = l1;
          } else if (jj & 1) {
            h1v = l1;
          } else {
            Y = (y - 2) >> 1;
            v2 = reduce3p(weightsAt(ay2, Y), h0v, h1v, l1);
            h0v = l1;
            emit = true;
          }
        } else {
          if ((jj & 1) == 0) {
            h0v = l1;
          } else {
            Y = (y - 1) >> 1;
            v2 = reduce2p(h0v, l1);
            emit = true;
          }
        }
        if (emit) {
          const float4 n1 = shflDown(v2, 1);
          const float4 o = TX1 ? reduce3p(wX, v2, n1, shflDown(v2, 2)) : reduce2p(v2, n1);
          storeIf(store2x, p.dst2 + uint64_t(Y) * p.pitch2 + uint64_t(X) * 4, encodeTexel(o, L));
        }
      }
    }
  };

  // two row buffers in turn: the next group's rows load while this one reduces
  uint32_t bufA[ROWS][4], bufB[ROWS][4];
  ldGroup(yb, bufA);
  for (uint32_t yg = yb;;) {
    if (yg + ROWS < ye) ldGroup(yg + ROWS, bufB);
    process(yg, bufA);
    yg += ROWS;
    if (yg >= ye) break;
    if (yg + ROWS < ye) ldGroup(yg + ROWS, bufA);
    process(yg, bufB);
    yg += ROWS;
    if (yg >= ye) break;
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

// Fill the aligned tables in `smem` (kAlignedLutSmemBytes of dynamic shared
// memory) and return the lane's table constants.  Call with every thread of
// the CTA; a __syncthreads must follow before the first lookup.
__device__ __forceinline__ Lut fillAlignedLut(uint8_t* smem, uint32_t tid, uint32_t nthreads) {
  const uint32_t base = smemAddr(smem);
  const uint32_t decOff = (0x10000u - (base & 0xFFFFu)) & 0xFFFFu;
  const uint32_t thrOff = decOff >= kLutThrBytes ? 0u : decOff + kLutDecodeBytes;
  fillLut(reinterpret_cast<float*>(smem + decOff), reinterpret_cast<float*>(smem + thrOff), tid, nthreads);
  Lut L = makeLutAt(base + decOff, base + thrOff, tid & 31);
  L.laneWord |= (base + decOff) & 0xFFFF0000u;  // table bytes 2-3 for decodeAligned
  return L;
}

}  // namespace
}  // namespace nvpyr
