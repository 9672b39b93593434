// kernels_tma.cu -- the sRGBA8 fast pipeline (nvpro_pyramid.glsl:209-534) for
// GB300: persistent CTAs, TMA tile loads, shuffle reductions, and the small
// trailing dispatches of a chain finished inside the same kernel.
//
// Work decomposition.  Level L of a fast dispatch with n levels is cut into
// 64x64 regions (each a whole number of the reference's 2^n tiles).  A CTA
// (512 threads, one per SM) holds four tile groups of four warps; each group
// owns a two-slot ring of 16 KiB region buffers filled by
// cp.async.bulk.tensor.2d (TMA) and completed on an mbarrier.  Inside a
// region, warp w of the group handles source rows 16w..16w+15:
//   level L+1: lane (cx = lane & 15, half = lane >> 4) reduces two 2x2 blocks
//              per row pair -> 8 texels, stored as 8-byte pairs;
//   level L+2: the half-warps exchange row pairs (shfl.xor 16), 2 texels/lane;
//   level L+3: horizontal neighbours via shfl.down 1;
//   level L+4: shfl.xor 16 + shfl.down 2;
//   level L+5/L+6: the group's 4x4 level-L+4 block goes through shared
//              memory and one warp (rotating per region) finishes it.
// The operand order of every REDUCE4 follows fastVerticalFirst(n, k), so the
// bytes equal the portable kernel's and the CPU oracle's.
//
// sRGB codec.  Decode is a table lookup per channel from a table replicated
// once per lane (row c holds 32 copies of decode[c] then 32 of alpha[c]), so
// a warp's 32 random lookups hit 32 distinct banks; the address is one PRMT.
// Encode computes a candidate code from lg2/ex2 (error well below 0.5 code)
// and corrects it with one comparison against the exact threshold table
// (also replicated per lane); the result equals the exact threshold count.
//
// Tail fusion.  When the dispatches after this one are small fast
// dispatches of the same image (e.g. F6 F2 after the first F6 of 16384^2),
// every CTA increments a counter after its regions; the last CTA (it sees
// count == gridDim.x - 1 after a release/acquire fence pair) runs those
// dispatches itself, reading the freshly written level with L2-coherent
// loads.  No thread waits on another CTA, so there is no spin on a flag.
#include <cuda.h>

#include <atomic>
#include <mutex>

#include "device_common.cuh"

namespace nvpyr {
namespace {

constexpr uint32_t kTile = 64;
constexpr uint32_t kGroups = 4;
constexpr uint32_t kGroupThreads = 128;
constexpr uint32_t kThreads = kGroups * kGroupThreads;
constexpr uint32_t kStages = 2;
constexpr uint32_t kTileBytes = kTile * kTile * 4;
constexpr uint32_t kMaxFused = 4;
constexpr uint32_t kWaitLimit = 1u << 22;  // bounded mbarrier polling

// Byte offsets inside the dynamic shared memory block.
constexpr uint32_t kLutDecodeOff = 0;                          // 256 rows x 256 B
constexpr uint32_t kLutThrOff = kLutDecodeOff + 256 * 256;     // 256 rows x 128 B
constexpr uint32_t kStageOff = kLutThrOff + 256 * 128;         // [group][stage] x 16 KiB
constexpr uint32_t kXchgOff = kStageOff + kGroups * kStages * kTileBytes;  // [group][2][16] float4
constexpr uint32_t kBarOff = kXchgOff + kGroups * 2 * 16 * 16;             // [group][stage] mbarrier
constexpr uint32_t kFlagOff = kBarOff + kGroups * kStages * 8;
constexpr uint32_t kSmemBytes = kFlagOff + 16;

struct FusedStage {
  uint32_t n;
  uint32_t coverW, coverH;  // covered extent of level L: multiples of 2^n
  uint32_t regionsX, regionsY;
  uint32_t l1Pairs;  // level L+1 accepts 8-byte stores
  const uint8_t* src;
  uint64_t srcPitch;
  uint8_t* dst[kMaxDispatchLevels + 1];
  uint64_t pitch[kMaxDispatchLevels + 1];
};

struct TmaParams {
  FusedStage st[kMaxFused];
  uint32_t stageCount;
  uint32_t* counter;    // last-CTA-done counter (self-resetting)
  uint32_t* errorFlag;  // set to 1 if a bounded wait gave up
};

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void groupSync(uint32_t g) {
  asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(kGroupThreads) : "memory");
}

__device__ __forceinline__ bool mbarWait(uint32_t bar, uint32_t parity) {
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tmaLoadRegion(uint32_t dst, const CUtensorMap* map, uint32_t x, uint32_t y,
                                              uint32_t bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kTileBytes) : "memory");
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
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

// Lane constants for the replicated tables.
struct Lut {
  uint32_t laneWord;  // byte0 = 4*lane, byte1 = 4*lane + 128 (alpha half of a row)
  uint32_t thrBase;   // kLutThrOff + 4*lane - (0x4B400000 << 7)  (see encodeChannel)
};

__device__ __forceinline__ float lutLoad(uint32_t byteOff) {
  extern __shared__ __align__(128) uint8_t smem[];
  return *reinterpret_cast<const float*>(smem + byteOff);
}

// NVPRO_PYRAMID_LOAD of one sRGBA8 texel: decode[r], decode[g], decode[b], alpha[a].
__device__ __forceinline__ float4 decodeTexel(uint32_t w, const Lut& L) {
  // PRMT builds (code << 8) | laneByte: row = code, column = this lane's copy.
  return make_float4(lutLoad(kLutDecodeOff + __byte_perm(w, L.laneWord, 0x6604)),
                     lutLoad(kLutDecodeOff + __byte_perm(w, L.laneWord, 0x6614)),
                     lutLoad(kLutDecodeOff + __byte_perm(w, L.laneWord, 0x6624)),
                     lutLoad(kLutDecodeOff + __byte_perm(w, L.laneWord, 0x6635)));
}

// Exact sRGB code of x (x >= 0, finite), returned in the low byte.
//   z = max(269.025 x^(5/12) - 14.525, min(3294.6 x - 0.5, 9.8)) approximates
//   255 * OETF(x) + 0.5 - 1 to ~1e-3, so a = rn(max(z, 0)) is code-1 or code;
//   code = a + (x >= threshold[a]).  The magic add leaves a in the low bits
//   of `bits`, and (bits << 7) + thrBase is the address of threshold[a].
__device__ __forceinline__ uint32_t encodeChannel(float x, const Lut& L) {
  const float p = ex2Approx(lg2Approx(x) * 0.41666666f);
  const float zp = fmaf(p, 269.025f, -14.525f);
  const float zl = fminf(fmaf(x, 3294.6f, -0.5f), 9.8f);
  const float z = fmaxf(fmaxf(zp, zl), 0.0f);
  const uint32_t bits = __float_as_uint(z + 12582912.0f);
  const float thr = lutLoad(bits * 128u + L.thrBase);
  return bits + (x >= thr ? 1u : 0u);
}

// srgbFromLinearVec's alpha: uint(a * 255 + 0.5) with truncation, via a
// round-toward-zero add that leaves the integer in the low mantissa bits.
__device__ __forceinline__ uint32_t encodeAlpha(float a) {
  const float s = __fadd_rn(__fmul_rn(a, 255.0f), 0.5f);
  return __float_as_uint(__fadd_rz(s, 8388608.0f));
}

__device__ __forceinline__ uint32_t encodeTexel(float4 v, const Lut& L) {
  const uint32_t r = encodeChannel(v.x, L), g = encodeChannel(v.y, L), b = encodeChannel(v.z, L);
  const uint32_t a = encodeAlpha(v.w);
  return __byte_perm(__byte_perm(r, g, 0x0040), __byte_perm(b, a, 0x0040), 0x5410);
}

__device__ __forceinline__ float4 shflXor(float4 v, int m) {
  return make_float4(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m),
                     __shfl_xor_sync(0xffffffffu, v.z, m), __shfl_xor_sync(0xffffffffu, v.w, m));
}
__device__ __forceinline__ float4 shflDown(float4 v, int d) {
  return make_float4(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d),
                     __shfl_down_sync(0xffffffffu, v.z, d), __shfl_down_sync(0xffffffffu, v.w, d));
}

__device__ __forceinline__ float4 sel4(bool c, float4 a, float4 b) { return c ? a : b; }

__device__ __forceinline__ void storeTexel(const FusedStage& st, uint32_t k, uint32_t x, uint32_t y, uint32_t v,
                                           bool check) {
  if (check && (x >= (st.coverW >> k) || y >= (st.coverH >> k))) return;
  *reinterpret_cast<uint32_t*>(st.dst[k] + y * st.pitch[k] + uint64_t(x) * 4) = v;
}

// Levels L+1..L+N of one 64x64 region whose texels are in `tile` (shared).
template <uint32_t N>
__device__ __forceinline__ void processRegion(const FusedStage& st, uint32_t region, const uint32_t* tile,
                                              float4* xchg, uint32_t g, uint32_t wig, uint32_t lane,
                                              uint32_t iter, const Lut& L) {
  const uint32_t x0 = (region % st.regionsX) * kTile, y0 = (region / st.regionsX) * kTile;
  const bool check = x0 + kTile > st.coverW || y0 + kTile > st.coverH;
  const uint32_t cx = lane & 15, half = lane >> 4;

  // ---- level L+1 (vertical pairs first, LOAD_REDUCE4) ----
  float4 a[4], b[4];
#pragma unroll
  for (uint32_t i = 0; i < 4; ++i) {
    const uint32_t r0 = 16 * wig + 4 * i + 2 * half;
    const uint4 t0 = reinterpret_cast<const uint4*>(tile + r0 * kTile)[cx];
    const uint4 t1 = reinterpret_cast<const uint4*>(tile + (r0 + 1) * kTile)[cx];
    a[i] = reduce4(decodeTexel(t0.x, L), decodeTexel(t1.x, L), decodeTexel(t0.y, L), decodeTexel(t1.y, L));
    b[i] = reduce4(decodeTexel(t0.z, L), decodeTexel(t1.z, L), decodeTexel(t0.w, L), decodeTexel(t1.w, L));
    const uint32_t ea = encodeTexel(a[i], L), eb = encodeTexel(b[i], L);
    const uint32_t X = (x0 >> 1) + 2 * cx, Y = (y0 >> 1) + 8 * wig + 2 * i + half;
    if (!check && st.l1Pairs) {
      *reinterpret_cast<uint2*>(st.dst[1] + Y * st.pitch[1] + uint64_t(X) * 4) = make_uint2(ea, eb);
    } else {
      storeTexel(st, 1, X, Y, ea, check);
      storeTexel(st, 1, X + 1, Y, eb, check);
    }
  }
  if (N < 2) return;

  // ---- level L+2: half 0 takes rows i = 0,1, half 1 rows i = 2,3 ----
  float4 c[2];
  {
    const float4 s0a = shflXor(sel4(half, a[0], a[2]), 16), s0b = shflXor(sel4(half, b[0], b[2]), 16);
    const float4 s1a = shflXor(sel4(half, a[1], a[3]), 16), s1b = shflXor(sel4(half, b[1], b[3]), 16);
    const bool vert = fastVerticalFirst(N, 2);
#pragma unroll
    for (uint32_t j = 0; j < 2; ++j) {
      const float4 ta = half ? (j ? s1a : s0a) : a[j], tb = half ? (j ? s1b : s0b) : b[j];
      const float4 ba = half ? a[2 + j] : (j ? s1a : s0a), bb = half ? b[2 + j] : (j ? s1b : s0b);
      c[j] = fastReduce(vert, ta, tb, ba, bb);
      storeTexel(st, 2, (x0 >> 2) + cx, (y0 >> 2) + 4 * wig + 2 * half + j, encodeTexel(c[j], L), check);
    }
  }
  if (N < 3) return;

  // ---- level L+3: row 2*wig + half; right neighbour in lane + 1 ----
  const float4 r0 = shflDown(c[0], 1), r1 = shflDown(c[1], 1);
  const float4 d = fastReduce(fastVerticalFirst(N, 3), c[0], r0, c[1], r1);
  if ((cx & 1) == 0)
    storeTexel(st, 3, (x0 >> 3) + (cx >> 1), (y0 >> 3) + 2 * wig + half, encodeTexel(d, L), check);
  if (N < 4) return;

  // ---- level L+4: row wig from rows 2*wig (half 0) and 2*wig+1 (half 1) ----
  const float4 e = shflXor(d, 16);
  const float4 dr = shflDown(d, 2), er = shflDown(e, 2);
  const float4 f = fastReduce(fastVerticalFirst(N, 4), d, dr, e, er);
  if (half == 0 && (cx & 3) == 0) {
    storeTexel(st, 4, (x0 >> 4) + (cx >> 2), (y0 >> 4) + wig, encodeTexel(f, L), check);
    if (N >= 5) xchg[wig * 4 + (cx >> 2)] = f;
  }
  if (N < 5) return;

  // ---- levels L+5, L+6 from the group's 4x4 block ----
  groupSync(g);
  if (wig == (iter & 3) && lane < 4) {
    const uint32_t px = lane & 1, py = lane >> 1;
    const float4 tl = xchg[(2 * py) * 4 + 2 * px], tr = xchg[(2 * py) * 4 + 2 * px + 1];
    const float4 bl = xchg[(2 * py + 1) * 4 + 2 * px], br = xchg[(2 * py + 1) * 4 + 2 * px + 1];
    const float4 v5 = fastReduce(fastVerticalFirst(N, 5), tl, tr, bl, br);
    storeTexel(st, 5, (x0 >> 5) + px, (y0 >> 5) + py, encodeTexel(v5, L), check);
    if (N >= 6) {
      const float4 v1 = make_float4(__shfl_xor_sync(0xfu, v5.x, 1), __shfl_xor_sync(0xfu, v5.y, 1),
                                    __shfl_xor_sync(0xfu, v5.z, 1), __shfl_xor_sync(0xfu, v5.w, 1));
      const float4 v2 = make_float4(__shfl_xor_sync(0xfu, v5.x, 2), __shfl_xor_sync(0xfu, v5.y, 2),
                                    __shfl_xor_sync(0xfu, v5.z, 2), __shfl_xor_sync(0xfu, v5.w, 2));
      const float4 v3 = make_float4(__shfl_xor_sync(0xfu, v5.x, 3), __shfl_xor_sync(0xfu, v5.y, 3),
                                    __shfl_xor_sync(0xfu, v5.z, 3), __shfl_xor_sync(0xfu, v5.w, 3));
      if (lane == 0)
        storeTexel(st, 6, x0 >> 6, y0 >> 6, encodeTexel(fastReduce(fastVerticalFirst(N, 6), v5, v1, v2, v3), L),
                   check);
    }
  }
}

__device__ __forceinline__ void processRegionN(const FusedStage& st, uint32_t region, const uint32_t* tile,
                                               float4* xchg, uint32_t g, uint32_t wig, uint32_t lane,
                                               uint32_t iter, const Lut& L) {
  switch (st.n) {
    case 1: processRegion<1>(st, region, tile, xchg, g, wig, lane, iter, L); break;
    case 2: processRegion<2>(st, region, tile, xchg, g, wig, lane, iter, L); break;
    case 3: processRegion<3>(st, region, tile, xchg, g, wig, lane, iter, L); break;
    case 4: processRegion<4>(st, region, tile, xchg, g, wig, lane, iter, L); break;
    case 5: processRegion<5>(st, region, tile, xchg, g, wig, lane, iter, L); break;
    default: processRegion<6>(st, region, tile, xchg, g, wig, lane, iter, L); break;
  }
}

// Fill a region buffer from global memory with L2-coherent loads (tail
// dispatches read a level written earlier in this kernel).  Texels outside
// the covered extent are zero, as the TMA fill would give.
__device__ __forceinline__ void loadRegionPlain(const FusedStage& st, uint32_t region, uint32_t* tile,
                                                uint32_t gtid) {
  const uint32_t x0 = (region % st.regionsX) * kTile, y0 = (region / st.regionsX) * kTile;
  for (uint32_t i = gtid; i < kTile * kTile; i += kGroupThreads) {
    const uint32_t x = i % kTile, y = i / kTile;
    uint32_t v = 0;
    if (x0 + x < st.coverW && y0 + y < st.coverH)
      v = __ldcg(reinterpret_cast<const unsigned int*>(st.src + uint64_t(y0 + y) * st.srcPitch +
                                                       uint64_t(x0 + x) * 4));
    tile[i] = v;
  }
}

__global__ void __launch_bounds__(kThreads, 1)
    tmaFastKernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ TmaParams p) {
  extern __shared__ __align__(128) uint8_t smem[];
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t g = warp >> 2, wig = warp & 3, gtid = tid & (kGroupThreads - 1);

  float* lutDec = reinterpret_cast<float*>(smem + kLutDecodeOff);
  float* lutThr = reinterpret_cast<float*>(smem + kLutThrOff);
  for (uint32_t i = tid; i < 256 * 32; i += kThreads) {
    const uint32_t code = i >> 5, l = i & 31;
    lutDec[code * 64 + l] = __uint_as_float(c_srgbDecodeBits[code]);
    lutDec[code * 64 + 32 + l] = __uint_as_float(c_alphaDecodeBits[code]);
    lutThr[code * 32 + l] = __uint_as_float(c_srgbThresholdBits[code]);
  }
  uint32_t* stage0 = reinterpret_cast<uint32_t*>(smem + kStageOff + (g * kStages + 0) * kTileBytes);
  uint32_t* stage1 = reinterpret_cast<uint32_t*>(smem + kStageOff + (g * kStages + 1) * kTileBytes);
  float4* xchgBase = reinterpret_cast<float4*>(smem + kXchgOff + g * 2 * 16 * 16);
  const uint32_t bar0 = smemAddr(smem + kBarOff + (g * kStages + 0) * 8);
  const uint32_t bar1 = bar0 + 8;
  uint32_t* flags = reinterpret_cast<uint32_t*>(smem + kFlagOff);
  if (gtid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  Lut L;
  L.laneWord = (4 * lane) | ((4 * lane + 128) << 8);
  L.thrBase = kLutThrOff + 4 * lane - (0x4B400000u << 7);

  const FusedStage& s0 = p.st[0];
  const uint32_t regions = s0.regionsX * s0.regionsY;
  const uint32_t G = gridDim.x * kGroups;
  const uint32_t gid = g * gridDim.x + blockIdx.x;
  if (gtid == 0) {
    for (uint32_t s = 0; s < kStages; ++s) {
      const uint32_t r = gid + s * G;
      if (r < regions)
        tmaLoadRegion(smemAddr(s ? stage1 : stage0), &tmap, (r % s0.regionsX) * kTile, (r / s0.regionsX) * kTile,
                      s ? bar1 : bar0);
    }
  }
  bool ok = true;
  uint32_t iter = 0;
  for (;; ++iter) {
    const uint32_t r = gid + iter * G;
    if (r >= regions) break;
    const uint32_t s = iter & 1;
    if (!mbarWait(s ? bar1 : bar0, (iter >> 1) & 1)) {
      ok = false;
      break;
    }
    processRegionN(s0, r, s ? stage1 : stage0, xchgBase + (iter & 1) * 16, g, wig, lane, iter, L);
    groupSync(g);  // every warp is done with this buffer
    const uint32_t rn = r + kStages * G;
    if (gtid == 0 && rn < regions)
      tmaLoadRegion(smemAddr(s ? stage1 : stage0), &tmap, (rn % s0.regionsX) * kTile, (rn / s0.regionsX) * kTile,
                    s ? bar1 : bar0);
  }
  if (!ok) {
    // A load never completed: record it, drain the other buffer (bounded) and
    // leave without touching the tail.
    if (gtid == 0) atomicExch(p.errorFlag, 1u);
    const uint32_t r1 = gid + (iter + 1) * G;
    if (r1 < regions) mbarWait(((iter + 1) & 1) ? bar1 : bar0, ((iter + 1) >> 1) & 1);
    return;
  }
  if (p.stageCount < 2) return;

  // ---- last CTA runs the trailing dispatches ----
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const uint32_t old = atomicAdd(p.counter, 1u);
    const uint32_t last = old == gridDim.x - 1;
    if (last) {
      *p.counter = 0;
      __threadfence();
    }
    flags[0] = last;
  }
  __syncthreads();
  if (!flags[0]) return;
  for (uint32_t d = 1; d < p.stageCount; ++d) {
    const FusedStage& st = p.st[d];
    const uint32_t nreg = st.regionsX * st.regionsY;
    for (uint32_t r = g, it = 0; r < nreg; r += kGroups, ++it) {
      loadRegionPlain(st, r, stage0, gtid);
      groupSync(g);
      processRegionN(st, r, stage0, xchgBase + (it & 1) * 16, g, wig, lane, it, L);
      groupSync(g);
    }
    __syncthreads();
  }
}

// Encode every float of x (test support for the exhaustive codec check).
__global__ void debugEncodeKernel(const float* x, uint8_t* fast, uint8_t* exact, uint64_t n) {
  extern __shared__ __align__(128) uint8_t smem[];
  float* lutThr = reinterpret_cast<float*>(smem + kLutThrOff);
  for (uint32_t i = threadIdx.x; i < 256 * 32; i += blockDim.x)
    lutThr[i] = __uint_as_float(c_srgbThresholdBits[i >> 5]);
  __syncthreads();
  Lut L;
  L.laneWord = 0;
  L.thrBase = kLutThrOff + 4 * (threadIdx.x & 31) - (0x4B400000u << 7);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const float v = x[i];
    fast[i] = uint8_t(encodeChannel(v, L));
    uint32_t c = 0;  // the oracle's threshold count (binary search)
    for (uint32_t step = 128; step > 0; step >>= 1)
      if (c + step <= 255 && lutThr[(c + step - 1) * 32] <= v) c += step;
    exact[i] = uint8_t(c);
  }
}

// ---------------------------------------------------------------------------
// Host side.

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encodeTiled() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return EncodeTiledFn(nullptr);
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

struct DeviceInfo {
  int sms = 0;
  bool configured = false;
};

cudaError_t deviceInfo(DeviceInfo** out) {
  static DeviceInfo infos[64];
  static std::mutex mu;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  DeviceInfo& d = infos[dev];
  if (!d.configured) {
    e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(tmaFastKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemBytes));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(debugEncodeKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemBytes));
    if (e != cudaSuccess) return e;
    d.configured = true;
  }
  *out = &d;
  return cudaSuccess;
}

uint64_t fastGroupsNeeded(const DispatchParams& p) {
  const uint32_t n = p.levelCount;
  const uint64_t tiles = uint64_t(p.lv[0].w >> n) * (p.lv[0].h >> n);
  const uint64_t perGroup = std::max<uint64_t>((n > 5 ? 4096u : 1024u) >> (2 * n), 1);
  return (tiles + perGroup - 1) / perGroup;
}

void fillStage(const DispatchParams& p, FusedStage* st) {
  const uint32_t n = p.levelCount;
  st->n = n;
  st->coverW = (p.lv[0].w >> n) << n;
  st->coverH = (p.lv[0].h >> n) << n;
  st->regionsX = (st->coverW + kTile - 1) / kTile;
  st->regionsY = (st->coverH + kTile - 1) / kTile;
  st->l1Pairs = (reinterpret_cast<uintptr_t>(p.lv[1].ptr) % 8 == 0) && (p.lv[1].pitch % 8 == 0);
  st->src = p.lv[0].ptr;
  st->srcPitch = p.lv[0].pitch;
  for (uint32_t k = 0; k <= kMaxDispatchLevels; ++k) {
    st->dst[k] = k <= n ? p.lv[k].ptr : nullptr;
    st->pitch[k] = k <= n ? p.lv[k].pitch : 0;
  }
}

}  // namespace

bool tmaFastSupported(const DispatchParams& p) {
  if (p.preset != kSrgba8 || !p.isFast || p.levelCount < 1 || p.levelCount > 6) return false;
  const LevelView& v = p.lv[0];
  if (reinterpret_cast<uintptr_t>(v.ptr) % 16 || v.pitch % 16 || v.pitch >= (uint64_t(1) << 40)) return false;
  if ((v.w >> p.levelCount) == 0 || (v.h >> p.levelCount) == 0) return false;
  if (p.groups < fastGroupsNeeded(p)) return false;  // partial grids: portable kernel
  return encodeTiled() != nullptr;
}

bool tmaTailCompatible(const DispatchParams& prev, const DispatchParams& next) {
  if (next.preset != kSrgba8 || !next.isFast || next.levelCount < 1 || next.levelCount > 6) return false;
  if (next.inputLevel != prev.inputLevel + prev.levelCount) return false;
  if (next.lv[0].ptr != prev.lv[prev.levelCount].ptr || next.lv[0].pitch != prev.lv[prev.levelCount].pitch)
    return false;
  if ((next.lv[0].w >> next.levelCount) == 0 || (next.lv[0].h >> next.levelCount) == 0) return false;
  if (next.groups < fastGroupsNeeded(next)) return false;
  // one CTA runs the tail: keep it to a few regions
  return uint64_t(next.lv[0].w) * next.lv[0].h <= 256u * 256u;
}

uint32_t tmaMaxFused() { return kMaxFused; }

cudaError_t launchTmaFast(const DispatchParams& p, const DispatchParams* tail, uint32_t tailCount,
                          cudaStream_t stream, const Scratch& scratch, uint32_t* launches) {
  DeviceInfo* info = nullptr;
  cudaError_t e = deviceInfo(&info);
  if (e != cudaSuccess) return e;
  if (tailCount + 1 > kMaxFused || (tailCount && scratch.counterCount < 2)) return cudaErrorInvalidValue;
  TmaParams tp{};
  fillStage(p, &tp.st[0]);
  for (uint32_t i = 0; i < tailCount; ++i) fillStage(tail[i], &tp.st[i + 1]);
  tp.stageCount = 1 + tailCount;
  tp.counter = scratch.counters;
  tp.errorFlag = scratch.counters ? scratch.counters + 1 : nullptr;

  CUtensorMap map;
  const cuuint64_t dims[2] = {p.lv[0].w, p.lv[0].h};
  const cuuint64_t strides[1] = {p.lv[0].pitch};
  const cuuint32_t box[2] = {kTile, kTile};
  const cuuint32_t estr[2] = {1, 1};
  CUresult cr = encodeTiled()(&map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, p.lv[0].ptr, dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return cudaErrorInvalidValue;
  const uint64_t regions = uint64_t(tp.st[0].regionsX) * tp.st[0].regionsY;
  const uint32_t grid = uint32_t(std::min<uint64_t>(regions, uint64_t(info->sms)));
  tmaFastKernel<<<grid, kThreads, kSmemBytes, stream>>>(map, tp);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launchDebugEncode(const float* x, uint8_t* fast, uint8_t* exact, uint64_t n, cudaStream_t stream) {
  DeviceInfo* info = nullptr;
  cudaError_t e = deviceInfo(&info);
  if (e != cudaSuccess) return e;
  debugEncodeKernel<<<info->sms * 2, 256, kSmemBytes, stream>>>(x, fast, exact, n);
  return cudaGetLastError();
}

}  // namespace nvpyr
