// kernels_tma.cu -- the sRGBA8 fast pipeline (nvpro_pyramid.glsl:209-534) for
// GB300: persistent CTAs, TMA tile loads, shuffle reductions, and the small
// trailing dispatches of a chain finished inside the same kernel.
//
// Work decomposition.  Level L of a fast dispatch with n levels is cut into
// 64x64 regions (each a whole number of the reference's 2^n tiles).  A CTA
// (512 threads, one per SM) holds four tile groups of four warps; each group
// owns a two-slot ring of 16 KiB region buffers filled by
// cp.async.bulk.tensor.2d (TMA) and completed on an mbarrier.  Inside a
// region, lane (cx = lane & 15, half = lane >> 4) of warp w of the group
// owns level-(L+1) rows 8w + 4half + i (i = 0..3), columns 2cx and 2cx+1:
//   level L+1: two 2x2 blocks per row pair of the buffer (LOAD_REDUCE4);
//   level L+2: from the lane's own row pairs, 2 texels per lane;
//   level L+3: horizontal neighbours via shfl.down 1;
//   level L+4: shfl.xor 16 + shfl.down 2;
//   level L+5/L+6: the group's 4x4 block of level L+4 goes through shared
//              memory to the last warp to deposit its part.
// The operand order of every REDUCE4 follows fastVerticalFirst(n, k), so the
// bytes equal the portable kernel's and the CPU oracle's.
//
// Producer warps.  Each group has a producer warp.  For each region i of
// its group it waits on the "buffer empty" mbarrier (four warp arrivals after
// their level-(L+1) reads) and issues the TMA of region i+2 into the buffer;
// then it waits on the "exchange full" mbarrier (four arrivals after the
// level-(L+4) deposits), finishes levels L+5/L+6 and arrives on the slot's
// "exchange empty" mbarrier, which the group waits on before depositing into
// that slot again (region i+2).  Consumer warps never wait on each other.
//
// sRGB codec.  Decode is a table lookup per channel from a table replicated
// once per lane (row c holds 32 copies of decode[c] then 32 of alpha[c]), so
// a warp's 32 random lookups hit 32 distinct banks; the address is one PRMT.
// Encode computes a candidate code from lg2/ex2 and corrects it with one
// comparison against the exact threshold table (also replicated per lane);
// the result equals the exact threshold count for every x in [0, 1].
//
// Trailing dispatches.  The small dispatches after this one (input levels of
// at most kSmallMaxTexels texels, fast or general: e.g. the F6 of the 64x64
// level after the first F6 of 4096^2, or everything after the F5 of
// 2560x1440) run in the same launch: every CTA increments a counter after
// its regions; the last CTA (it sees the count reach gridDim.x after a
// release/acquire fence pair) runs them with the small-dispatch engine
// (small_engine.cuh) in the freed region buffers.  No thread waits on another
// CTA, so there is no spin on a flag.  Every CTA arrives, also one whose
// bounded wait gave up (it then marks its arrival as failed and the last CTA
// skips the tail), so the counter is back at zero when the kernel ends,
// whatever happened.
#include <cuda.h>

#include <atomic>
#include <mutex>

#include "small_engine.cuh"

namespace nvpyr {
namespace {

constexpr uint32_t kTile = 64;
constexpr uint32_t kGroups = 4;
constexpr uint32_t kGroupWarps = 4;
constexpr uint32_t kGroupThreads = kGroupWarps * 32;
constexpr uint32_t kConsumerThreads = kGroups * kGroupThreads;
constexpr uint32_t kProducerWarp0 = kConsumerThreads / 32;  // one producer warp per group
constexpr uint32_t kThreads = kConsumerThreads + 32 * kGroups;
constexpr uint32_t kStages = 2;
constexpr uint32_t kXchgRing = 2;
constexpr uint32_t kTileBytes = kTile * kTile * 4;
// Bounded mbarrier waits: each try_wait carries a suspend-time hint, so a
// waiting warp is parked by the hardware until the phase completes (or the
// hint runs out) instead of polling.  After about a second of %globaltimer
// time, or kWaitPolls polls, the wait gives up and reports it.  (Measured on
// 16384^2: the F6 launch 285 -> 278 us against polling with nanosleep.)
constexpr uint32_t kSuspendHintNs = 20000;
constexpr uint32_t kWaitLimitNs = 1000000000u;
constexpr uint32_t kWaitPolls = 1u << 22;
// The timer is read every kPollsPerTimerRead polls (a power of two), not on
// every poll: waiting warps then take fewer issue slots from the working
// ones (16384^2 F6 launch 291 -> 287 us).
constexpr uint32_t kPollsPerTimerRead = 16;
// The producer warps' waits (buffer empty, exchange full) are off the
// consumers' critical path: between their polls they sleep, leaving the issue
// slots to the consumer warps.
constexpr uint32_t kProducerSleepNs = 256;
// Tail counter arrivals: the low 16 bits count CTAs (grids are at most one
// CTA per SM), a CTA whose wait gave up adds this as well.
constexpr uint32_t kFailedArrival = 1u << 16;

// Byte offsets inside the dynamic shared memory block.
constexpr uint32_t kLutDecodeOff = 0;                          // 256 rows x 256 B
constexpr uint32_t kLutThrOff = kLutDecodeOff + 256 * 256;     // 255 rows x 128 B
constexpr uint32_t kStageOff = kLutThrOff + kThrRows * 128;    // [group][stage] x 16 KiB
constexpr uint32_t kXchgOff = kStageOff + kGroups * kStages * kTileBytes;  // [group][ring][16] float4
constexpr uint32_t kBarOff = kXchgOff + kGroups * kXchgRing * 16 * 16;     // mbarriers, per group:
// full[stage], empty[stage], xfull[ring], xempty[ring]
constexpr uint32_t kBarsPerGroup = 2 * kStages + 2 * kXchgRing;
constexpr uint32_t kIssuedOff = kBarOff + kGroups * kBarsPerGroup * 8;  // [group][stage] TMA loads issued
constexpr uint32_t kSmemBytes = kIssuedOff + kGroups * kStages * 4;
static_assert(kStageOff % 128 == 0, "TMA destinations need 128-byte alignment");
static_assert(kSmemBytes <= 232448, "exceeds the 227 KiB of shared memory per CTA");
static_assert(kSmallArenaBytes <= kGroups * kStages * kTileBytes, "the tail runs in the region buffers");
constexpr uint32_t kDebugSmemBytes = kLutThrOff + kThrRows * 128;

struct FusedStage {
  uint32_t n;
  uint32_t coverW, coverH;  // covered extent of level L: multiples of 2^n
  uint32_t regionsX, regionsY;
  const uint8_t* src;
  uint64_t srcPitch;
  uint8_t* dst[kMaxDispatchLevels + 1];
  uint64_t pitch[kMaxDispatchLevels + 1];
};

struct TmaParams {
  FusedStage st;                            // the dispatch over the TMA-loaded level
  SmallDispatch tail[kMaxSmallDispatches];  // the small dispatches after it
  uint32_t tailCount;
  uint32_t* counter;    // last-CTA-done counter (self-resetting)
  uint32_t* errorFlag;  // set to 1 if a bounded wait gave up
  // Test support: this CTA gives up at once, as if its first wait had run out
  // (no CTA when out of range).
  uint32_t failCta;
};

__device__ __forceinline__ Lut makeLut(uint32_t lane) {
  extern __shared__ __align__(128) uint8_t smem[];
  const uint32_t base = smemAddr(smem);
  return makeLutAt(base + kLutDecodeOff, base + kLutThrOff, lane);
}

// Low 32 bits of the nanosecond global timer (wraps every ~4.3 s; the
// unsigned difference of two reads is exact for waits below that).
__device__ __forceinline__ uint32_t globalTimerLoNs() {
  uint32_t t;
  asm volatile("mov.u32 %0, %%globaltimer_lo;" : "=r"(t));
  return t;
}

// SLEEP_NS: after a poll that found the phase incomplete, the warp sleeps
// this long before the next (0: none).
template <uint32_t SLEEP_NS = 0>
__device__ __forceinline__ bool mbarWait(uint32_t bar, uint32_t parity) {
  uint32_t t0 = 0;
  for (uint32_t it = 0; it < kWaitPolls; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity), "r"(kSuspendHintNs)
        : "memory");
    if (done) return true;
    if (SLEEP_NS) __nanosleep(SLEEP_NS);
    if ((it & (kPollsPerTimerRead - 1)) != kPollsPerTimerRead - 1) continue;
    const uint32_t t = globalTimerLoNs();
    if (it == kPollsPerTimerRead - 1)
      t0 = t;
    else if (t - t0 > kWaitLimitNs)
      return false;
  }
  return false;
}

__device__ __forceinline__ void mbarArrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
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

__device__ __forceinline__ uint32_t* texelPtr(const FusedStage& st, uint32_t k, uint32_t x, uint32_t y) {
  return reinterpret_cast<uint32_t*>(st.dst[k] + y * st.pitch[k] + uint64_t(x) * 4);
}

// Store texel (x, y) of level L+k; edge regions (CHECK) skip texels outside
// the covered extent.
template <bool CHECK>
__device__ __forceinline__ void storeTexel(const FusedStage& st, uint32_t k, uint32_t x, uint32_t y, uint32_t v) {
  if (CHECK && (x >= (st.coverW >> k) || y >= (st.coverH >> k))) return;
  *texelPtr(st, k, x, y) = v;
}

// Levels L+1 and L+2 of a region from the buffer `tile`: the lane's four
// level-(L+1) rows are built two at a time, each pair giving one level-(L+2)
// texel (rows 4*wig + 2*half + j).  Level L+1 is stored as 8-byte pairs
// (2cx, 2cx+1).  Returns the two level-(L+2) values.
template <uint32_t N, bool CHECK>
__device__ __forceinline__ void levels12(const FusedStage& st, uint32_t x0, uint32_t y0, const uint32_t* tile,
                                         uint32_t wig, uint32_t lane, const Lut& L, float4& c0, float4& c1) {
  const uint32_t cx = lane & 15, half = lane >> 4;
  const uint32_t X = (x0 >> 1) + 2 * cx, Y0 = (y0 >> 1) + 8 * wig + 4 * half;
  uint8_t* row = st.dst[1] + uint64_t(Y0) * st.pitch[1] + uint64_t(X) * 4;
  const uint4* src = reinterpret_cast<const uint4*>(tile + (16 * wig + 8 * half) * kTile) + cx;
  const bool inX = !CHECK || X < (st.coverW >> 1);  // X even, covered width even: pairs are whole
#pragma unroll
  for (uint32_t j = 0; j < 2; ++j) {
    const uint4 t0 = src[0], t1 = src[kTile / 4], t2 = src[2 * kTile / 4], t3 = src[3 * kTile / 4];
    src += kTile;  // four rows of 64 texels
    const float4 a0 = reduce4p(decodeTexel(t0.x, L), decodeTexel(t1.x, L), decodeTexel(t0.y, L), decodeTexel(t1.y, L));
    const float4 b0 = reduce4p(decodeTexel(t0.z, L), decodeTexel(t1.z, L), decodeTexel(t0.w, L), decodeTexel(t1.w, L));
    const float4 a1 = reduce4p(decodeTexel(t2.x, L), decodeTexel(t3.x, L), decodeTexel(t2.y, L), decodeTexel(t3.y, L));
    const float4 b1 = reduce4p(decodeTexel(t2.z, L), decodeTexel(t3.z, L), decodeTexel(t2.w, L), decodeTexel(t3.w, L));
    const uint2 e0 = make_uint2(encodeTexel(a0, L), encodeTexel(b0, L));
    const uint2 e1 = make_uint2(encodeTexel(a1, L), encodeTexel(b1, L));
    const uint32_t Y = Y0 + 2 * j;
    if (!CHECK || (inX && Y < (st.coverH >> 1))) *reinterpret_cast<uint2*>(row) = e0;
    if (!CHECK || (inX && Y + 1 < (st.coverH >> 1))) *reinterpret_cast<uint2*>(row + st.pitch[1]) = e1;
    row += 2 * st.pitch[1];
    if (N >= 2) {
      const float4 c = fastReduceP(fastVerticalFirst(N, 2), a0, b0, a1, b1);
      storeTexel<CHECK>(st, 2, (x0 >> 2) + cx, (y0 >> 2) + 4 * wig + 2 * half + j, encodeTexel(c, L));
      if (j == 0)
        c0 = c;
      else
        c1 = c;
    }
  }
}

// Levels L+3 (row 2*wig + half, even cx) and L+4 (row wig, half 0,
// cx % 4 == 0) from the level-(L+2) values, encoded in one pass: the
// level-(L+4) value moves to the idle odd lane cx + 1, and each lane makes
// at most one store.  For N >= 5 the level-(L+4) values go to `xchg`
// ([row][col], 4x4).  SF: the pipeline's shared format, applied to the
// values handed on from level L+3 (N = 4, 5) or L+4 (N = 6); the level
// itself is stored from its FP32 values.
template <uint32_t N, uint32_t SF, bool CHECK>
__device__ __forceinline__ void levels34(const FusedStage& st, uint32_t x0, uint32_t y0, float4 c0, float4 c1,
                                         float4* xchg, uint32_t wig, uint32_t lane, const Lut& L) {
  if (N < 3) return;
  const uint32_t cx = lane & 15, half = lane >> 4;
  const float4 r0 = shflDown(c0, 1), r1 = shflDown(c1, 1);
  const float4 d = fastReduceP(fastVerticalFirst(N, 3), c0, r0, c1, r1);
  float4 v = d;
  // this lane's output: level L+3 texel (even cx) or level L+4 texel (odd cx)
  uint32_t k = 3, x = (x0 >> 3) + (cx >> 1), y = (y0 >> 3) + 2 * wig + half;
  bool store = (cx & 1) == 0;
  if (N >= 4) {
    const float4 dh = N <= 5 ? sharedRoundTrip<SF>(d, L) : d;
    const float4 e = shflXor(dh, 16);
    const float4 dr = shflDown(dh, 2), er = shflDown(e, 2);
    const float4 f = fastReduceP(fastVerticalFirst(N, 4), dh, dr, e, er);
    if (N >= 5 && half == 0 && (cx & 3) == 0) xchg[wig * 4 + (cx >> 2)] = N == 6 ? sharedRoundTrip<SF>(f, L) : f;
    const float4 fu = shflUp(f, 1);
    if (cx & 1) {
      v = fu;
      k = 4;
      x = (x0 >> 4) + (cx >> 2);
      y = (y0 >> 4) + wig;
      store = half == 0 && (cx & 3) == 1;
    }
  }
  const uint32_t code = encodeTexel(v, L);
  if (store) storeTexel<CHECK>(st, k, x, y, code);
}

// Levels L+5 (and L+6) of a region from the group's 4x4 block in `xchg`,
// by one warp: lanes 0..3 build level L+5, lane 4 receives level L+6; one
// encode pass.
template <uint32_t N, bool CHECK>
__device__ __forceinline__ void finishTop(const FusedStage& st, uint32_t x0, uint32_t y0, const float4* xchg,
                                          uint32_t lane, const Lut& L) {
  if (N < 5 || lane >= 8) return;
  const uint32_t px = lane & 1, py = (lane >> 1) & 1;
  const float4 tl = xchg[(2 * py) * 4 + 2 * px], tr = xchg[(2 * py) * 4 + 2 * px + 1];
  const float4 bl = xchg[(2 * py + 1) * 4 + 2 * px], br = xchg[(2 * py + 1) * 4 + 2 * px + 1];
  float4 v = fastReduceP(fastVerticalFirst(N, 5), tl, tr, bl, br);
  if (N >= 6) {
    constexpr uint32_t m = 0xffu;
    const float4 v1 = make_float4(__shfl_xor_sync(m, v.x, 1), __shfl_xor_sync(m, v.y, 1),
                                  __shfl_xor_sync(m, v.z, 1), __shfl_xor_sync(m, v.w, 1));
    const float4 v2 = make_float4(__shfl_xor_sync(m, v.x, 2), __shfl_xor_sync(m, v.y, 2),
                                  __shfl_xor_sync(m, v.z, 2), __shfl_xor_sync(m, v.w, 2));
    const float4 v3 = make_float4(__shfl_xor_sync(m, v.x, 3), __shfl_xor_sync(m, v.y, 3),
                                  __shfl_xor_sync(m, v.z, 3), __shfl_xor_sync(m, v.w, 3));
    const float4 top = fastReduceP(fastVerticalFirst(N, 6), v, v1, v2, v3);  // valid in lane 0
    const float4 t4 = make_float4(__shfl_sync(m, top.x, 0), __shfl_sync(m, top.y, 0), __shfl_sync(m, top.z, 0),
                                  __shfl_sync(m, top.w, 0));
    if (lane == 4) v = t4;
  }
  if (lane > 4 || (N < 6 && lane == 4)) return;
  const uint32_t code = encodeTexel(v, L);
  if (lane < 4)
    storeTexel<CHECK>(st, 5, (x0 >> 5) + px, (y0 >> 5) + py, code);
  else
    storeTexel<CHECK>(st, 6, x0 >> 6, y0 >> 6, code);
}

struct GroupCtx {
  const uint32_t* tiles;  // this group's region buffers
  uint32_t stage0;        // shared address of its first buffer
  uint32_t full0;         // mbarriers: full[stage], empty[stage], xfull[ring]
  uint32_t empty0;
  uint32_t xfull0;
  uint32_t xempty0;
  float4* xchg;           // this group's exchange ring
  uint32_t* issued;       // TMA loads issued per stage (producer lane 0 only)
};

__device__ __forceinline__ GroupCtx groupCtx(uint32_t g) {
  extern __shared__ __align__(128) uint8_t smem[];
  GroupCtx G;
  G.tiles = reinterpret_cast<const uint32_t*>(smem + kStageOff + g * kStages * kTileBytes);
  G.stage0 = smemAddr(G.tiles);
  G.full0 = smemAddr(smem + kBarOff + g * kBarsPerGroup * 8);
  G.empty0 = G.full0 + 8 * kStages;
  G.xfull0 = G.empty0 + 8 * kStages;
  G.xempty0 = G.xfull0 + 8 * kXchgRing;
  G.xchg = reinterpret_cast<float4*>(smem + kXchgOff) + g * kXchgRing * 16;
  G.issued = reinterpret_cast<uint32_t*>(smem + kIssuedOff) + g * kStages;
  return G;
}

// One region of the main (TMA-fed) loop for a consumer warp.
template <uint32_t N, uint32_t SF, bool CHECK>
__device__ __forceinline__ bool mainRegion(const FusedStage& st, const GroupCtx& G, uint32_t x0, uint32_t y0,
                                           uint32_t iter, uint32_t wig, uint32_t lane, const Lut& L) {
  const uint32_t s = iter & 1, ring = iter & 1;
  const uint32_t* tile = G.tiles + s * (kTileBytes / 4);
  float4 c0 = make_float4(0, 0, 0, 0), c1 = c0;
  levels12<N, CHECK>(st, x0, y0, tile, wig, lane, L, c0, c1);
  __syncwarp();
  if (lane == 0) mbarArrive(G.empty0 + 8 * s);  // this warp is done with the buffer
  // before depositing into this exchange slot again, the producer must have
  // finished the region that used it two steps ago
  if (N >= 5 && iter >= 2 && !mbarWait(G.xempty0 + 8 * ring, ((iter >> 1) - 1) & 1)) return false;
  levels34<N, SF, CHECK>(st, x0, y0, c0, c1, G.xchg + ring * 16, wig, lane, L);
  if (N >= 5) {
    __syncwarp();
    if (lane == 0) mbarArrive(G.xfull0 + 8 * ring);  // its part of the 4x4 block is deposited
  }
  return true;
}

// Region coordinates (in regions) of a group's i-th region, advanced by the
// stride of all groups without divisions.
struct RegionCursor {
  uint32_t rx, ry, dx, dy, RX;
  __device__ __forceinline__ RegionCursor(uint32_t first, uint32_t stride, uint32_t regionsX)
      : rx(first % regionsX), ry(first / regionsX), dx(stride % regionsX), dy(stride / regionsX), RX(regionsX) {}
  __device__ __forceinline__ void next() {
    rx += dx;
    ry += dy;
    if (rx >= RX) {
      rx -= RX;
      ++ry;
    }
  }
};

template <uint32_t N, uint32_t SF>
__device__ __forceinline__ bool consumerLoop(const FusedStage& st, const GroupCtx& G, uint32_t gid,
                                             uint32_t groupsTotal, uint32_t wig, uint32_t lane, const Lut& L) {
  RegionCursor c(gid, groupsTotal, st.regionsX);
  for (uint32_t iter = 0; c.ry < st.regionsY; ++iter, c.next()) {
    const uint32_t s = iter & 1;
    if (!mbarWait(G.full0 + 8 * s, (iter >> 1) & 1)) return false;
    const uint32_t x0 = c.rx * kTile, y0 = c.ry * kTile;
    const bool ok = (x0 + kTile > st.coverW || y0 + kTile > st.coverH)
                        ? mainRegion<N, SF, true>(st, G, x0, y0, iter, wig, lane, L)
                        : mainRegion<N, SF, false>(st, G, x0, y0, iter, wig, lane, L);
    if (!ok) return false;
  }
  return true;
}

// The shared format that applies to an N-level dispatch of a pipeline with
// format SF: only dispatches of 4 or more levels hand values on.
template <uint32_t N, uint32_t SF>
constexpr uint32_t kFmtOf = N >= 4 ? SF : kSharedFp32;

// The producer warp of group g: refill region i's buffer with region i+2 as
// soon as it is empty, then finish levels L+5/L+6 of region i.
template <uint32_t N>
__device__ __forceinline__ bool producerLoop(const FusedStage& st, const CUtensorMap* map, const GroupCtx& G,
                                             uint32_t gid, uint32_t groupsTotal, uint32_t lane, const Lut& L) {
  RegionCursor cur(gid, groupsTotal, st.regionsX);
  RegionCursor ahead = cur;
  ahead.next();
  ahead.next();
  for (uint32_t iter = 0; cur.ry < st.regionsY; ++iter, cur.next(), ahead.next()) {
    const uint32_t s = iter & 1, parity = (iter >> 1) & 1;
    if (ahead.ry < st.regionsY) {
      if (!mbarWait<kProducerSleepNs>(G.empty0 + 8 * s, parity)) return false;
      if (lane == 0) {
        tmaLoadRegion(G.stage0 + s * kTileBytes, map, ahead.rx * kTile, ahead.ry * kTile, G.full0 + 8 * s);
        ++G.issued[s];
      }
    }
    if (N >= 5) {
      if (!mbarWait<kProducerSleepNs>(G.xfull0 + 8 * s, parity)) return false;
      const uint32_t x0 = cur.rx * kTile, y0 = cur.ry * kTile;
      if (x0 + kTile > st.coverW || y0 + kTile > st.coverH)
        finishTop<N, true>(st, x0, y0, G.xchg + s * 16, lane, L);
      else
        finishTop<N, false>(st, x0, y0, G.xchg + s * 16, lane, L);
      __syncwarp();
      if (lane == 0) mbarArrive(G.xempty0 + 8 * s);  // the slot may be reused
    }
  }
  return true;
}

template <uint32_t SF>
__device__ __forceinline__ bool mainLoopN(const FusedStage& st, const CUtensorMap* map, uint32_t warp,
                                          uint32_t groupsTotal, uint32_t lane, const Lut& L) {
  if (warp >= kProducerWarp0) {
    const uint32_t g = warp - kProducerWarp0;
    const GroupCtx G = groupCtx(g);
    const uint32_t gid = g * gridDim.x + blockIdx.x;
    switch (st.n) {
      case 1: return producerLoop<1>(st, map, G, gid, groupsTotal, lane, L);
      case 2: return producerLoop<2>(st, map, G, gid, groupsTotal, lane, L);
      case 3: return producerLoop<3>(st, map, G, gid, groupsTotal, lane, L);
      case 4: return producerLoop<4>(st, map, G, gid, groupsTotal, lane, L);
      case 5: return producerLoop<5>(st, map, G, gid, groupsTotal, lane, L);
      default: return producerLoop<6>(st, map, G, gid, groupsTotal, lane, L);
    }
  }
  const uint32_t g = warp / kGroupWarps, wig = warp % kGroupWarps;
  const GroupCtx G = groupCtx(g);
  const uint32_t gid = g * gridDim.x + blockIdx.x;
  switch (st.n) {
    case 1: return consumerLoop<1, kFmtOf<1, SF>>(st, G, gid, groupsTotal, wig, lane, L);
    case 2: return consumerLoop<2, kFmtOf<2, SF>>(st, G, gid, groupsTotal, wig, lane, L);
    case 3: return consumerLoop<3, kFmtOf<3, SF>>(st, G, gid, groupsTotal, wig, lane, L);
    case 4: return consumerLoop<4, kFmtOf<4, SF>>(st, G, gid, groupsTotal, wig, lane, L);
    case 5: return consumerLoop<5, kFmtOf<5, SF>>(st, G, gid, groupsTotal, wig, lane, L);
    default: return consumerLoop<6, kFmtOf<6, SF>>(st, G, gid, groupsTotal, wig, lane, L);
  }
}

// SF: the fast pipeline's shared format (the same for every stage of a launch).
template <uint32_t SF>
__global__ void __launch_bounds__(kThreads, 1)
    tmaFastKernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ TmaParams p) {
  extern __shared__ __align__(128) uint8_t smem[];
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  fillLut(reinterpret_cast<float*>(smem + kLutDecodeOff), reinterpret_cast<float*>(smem + kLutThrOff), tid,
          kThreads);
  if (tid == 0) {
    for (uint32_t g = 0; g < kGroups; ++g) {
      const GroupCtx G = groupCtx(g);
      for (uint32_t s = 0; s < kStages; ++s) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(G.full0 + 8 * s) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(G.empty0 + 8 * s), "r"(kGroupWarps) : "memory");
      }
      for (uint32_t b = 0; b < kXchgRing; ++b) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(G.xfull0 + 8 * b), "r"(kGroupWarps) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(G.xempty0 + 8 * b) : "memory");
      }
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid < kGroups * kStages) reinterpret_cast<uint32_t*>(smem + kIssuedOff)[tid] = 0;
  __syncthreads();
  const Lut L = makeLut(lane);
  // Programmatic dependent launch: everything above (tables, barriers) may
  // overlap the end of the previous kernel on the stream; the first global
  // access waits here until that kernel has completed and its writes are
  // visible.  Then let the next kernel on the stream begin its own prologue
  // as SMs free up.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

  const FusedStage& s0 = p.st;
  const uint32_t regions = s0.regionsX * s0.regionsY;
  const uint32_t groupsTotal = gridDim.x * kGroups;
  if (warp >= kProducerWarp0 && lane == 0) {  // the first two regions of the group
    const uint32_t g = warp - kProducerWarp0;
    const GroupCtx G = groupCtx(g);
    for (uint32_t s = 0; s < kStages; ++s) {
      const uint32_t r = g * gridDim.x + blockIdx.x + s * groupsTotal;
      if (r < regions) {
        tmaLoadRegion(G.stage0 + s * kTileBytes, &tmap, (r % s0.regionsX) * kTile, (r / s0.regionsX) * kTile,
                      G.full0 + 8 * s);
        ++G.issued[s];
      }
    }
  }
  __syncwarp();
  const bool ok = blockIdx.x != p.failCta && mainLoopN<SF>(s0, &tmap, warp, groupsTotal, lane, L);
  const bool failed = __syncthreads_or(!ok);
  if (failed && tid == 0) {
    // A bounded wait gave up: record it, and wait (bounded) for the last load
    // issued into each buffer, which may still be in flight, before the CTA
    // may exit.  Load n of a buffer completes phase n - 1 of its mbarrier.
    atomicExch(p.errorFlag, 1u);
    for (uint32_t g = 0; g < kGroups; ++g) {
      const GroupCtx G = groupCtx(g);
      for (uint32_t s = 0; s < kStages; ++s)
        if (G.issued[s]) mbarWait(G.full0 + 8 * s, (G.issued[s] - 1) & 1);
    }
  }
  if (p.tailCount == 0) return;

  // ---- last CTA runs the trailing dispatches ----
  // Every CTA arrives, a failed one with kFailedArrival added, so the counter
  // always returns to zero (no later launch sees a partial count); the tail
  // is skipped when any CTA failed, since its input level is incomplete.
  uint32_t last = 0;
  if (tid == 0) {
    __threadfence();
    const uint32_t inc = failed ? kFailedArrival + 1 : 1u;
    const uint32_t total = atomicAdd(p.counter, inc) + inc;
    if ((total & (kFailedArrival - 1)) == gridDim.x) {
      *p.counter = 0;
      __threadfence();
      last = total < kFailedArrival;
    }
  }
  if (!__syncthreads_or(last)) return;
  // every thread of the CTA, the producer warps too, in the freed region buffers
  runSmallDispatches(p.tail, p.tailCount, smem + kStageOff, LutCodec{L}, tid, kThreads);
}

// Test support for failure detection: one warp waits, with the kernels' own
// bounded mbarrier wait, on a phase that nothing completes (no thread
// arrives); the wait gives up after its time limit and the error flag is set,
// as a stalled TMA load would leave it.  Nothing is in flight when it exits.
__global__ void debugMbarTimeoutKernel(uint32_t* errorFlag) {
  __shared__ __align__(8) uint64_t bar;
  const uint32_t addr = smemAddr(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(addr) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (threadIdx.x == 0 && !mbarWait(addr, 0)) atomicExch(errorFlag, 1u);
}

// Encode every float of x (test support for the exhaustive codec check).
// alpha = 0: the value goes through the packed texel encoder as colour
// channel i % 3, with its neighbours in the array as the other channels, and
// `exact` is the threshold count; alpha = 1: the value is the texel's alpha
// and `exact` is the scalar alphaEncode.
__global__ void debugEncodeKernel(const float* x, uint8_t* fast, uint8_t* exact, uint64_t n, uint32_t alpha) {
  extern __shared__ __align__(128) uint8_t smem[];
  float* lutThr = reinterpret_cast<float*>(smem + kLutThrOff);
  __shared__ float full[256];
  for (uint32_t i = threadIdx.x; i < kThrRows * 32; i += blockDim.x)
    lutThr[i] = __uint_as_float(c_srgbThresholdBits[i >> 5]);
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) full[i] = __uint_as_float(c_srgbThresholdBits[i]);
  __syncthreads();
  const Lut L = makeLut(threadIdx.x & 31);
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const float v = x[i];
    // The fast encoder's table index is derived from the value; keep it in
    // the encoder's domain [0, 1] (NaN -> 0) whatever the caller passes.
    auto dom = [](float f) { return fminf(fmaxf(f, 0.0f), 1.0f); };
    const float u = dom(x[(i + 1) % n]), w = dom(x[(i + 2) % n]), cv = dom(v);
    if (alpha) {
      fast[i] = uint8_t(encodeTexel(make_float4(u, w, u, cv), L) >> 24);
      exact[i] = uint8_t(alphaEncode(cv));
      continue;
    }
    const uint32_t ch = uint32_t(i % 3);
    const float4 t = ch == 0 ? make_float4(cv, u, w, 0.5f) : ch == 1 ? make_float4(u, cv, w, 0.5f)
                                                                    : make_float4(u, w, cv, 0.5f);
    fast[i] = uint8_t(encodeTexel(t, L) >> (8 * ch));
    uint32_t c = 0;  // the oracle's threshold count (binary search)
    for (uint32_t step = 128; step > 0; step >>= 1)
      if (c + step <= 255 && full[c + step - 1] <= v) c += step;
    exact[i] = uint8_t(c);
  }
}

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

const void* tmaKernel(uint32_t sharedFmt) {
  return sharedFmt == kSharedSrgb  ? reinterpret_cast<const void*>(tmaFastKernel<kSharedSrgb>)
         : sharedFmt == kSharedF16 ? reinterpret_cast<const void*>(tmaFastKernel<kSharedF16>)
                                   : reinterpret_cast<const void*>(tmaFastKernel<kSharedFp32>);
}

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
    for (const void* k : {tmaKernel(kSharedFp32), tmaKernel(kSharedSrgb), tmaKernel(kSharedF16)})
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemBytes));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(debugEncodeKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               int(kDebugSmemBytes));
    if (e != cudaSuccess) return e;
    d.configured = true;
  }
  *out = &d;
  return cudaSuccess;
}

void fillStage(const DispatchParams& p, FusedStage* st) {
  const uint32_t n = p.levelCount;
  st->n = n;
  st->coverW = (p.lv[0].w >> n) << n;
  st->coverH = (p.lv[0].h >> n) << n;
  st->regionsX = (st->coverW + kTile - 1) / kTile;
  st->regionsY = (st->coverH + kTile - 1) / kTile;
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
  // 8-byte level-(L+1) pairs: aligned, and whole at the right edge
  if (reinterpret_cast<uintptr_t>(p.lv[1].ptr) % 8 || p.lv[1].pitch % 8 || ((v.w >> p.levelCount) << p.levelCount) % 4)
    return false;
  if (p.groups < fastGroupsNeeded(p)) return false;  // partial grids: portable kernel
  return encodeTiled() != nullptr;
}

cudaError_t launchTmaFast(const DispatchParams& p, const DispatchParams* tail, uint32_t tailCount,
                          cudaStream_t stream, const Scratch& scratch, uint32_t* launches, uint32_t debugFailCta) {
  DeviceInfo* info = nullptr;
  cudaError_t e = deviceInfo(&info);
  if (e != cudaSuccess) return e;
  if (tailCount > kMaxSmallDispatches || (tailCount && scratch.counterCount < kTmaScratchWords))
    return cudaErrorInvalidValue;
  // the tail's dispatches carry their own shared formats (the engine applies them)
  TmaParams tp{};
  fillStage(p, &tp.st);
  for (uint32_t i = 0; i < tailCount; ++i) makeSmallDispatch(tail[i], &tp.tail[i]);
  tp.tailCount = tailCount;
  tp.counter = scratch.counters;
  tp.errorFlag = scratch.counters ? scratch.error() : nullptr;
  tp.failCta = tp.errorFlag ? debugFailCta : ~0u;

  CUtensorMap map;
  const cuuint64_t dims[2] = {p.lv[0].w, p.lv[0].h};
  const cuuint64_t strides[1] = {p.lv[0].pitch};
  const cuuint32_t box[2] = {kTile, kTile};
  const cuuint32_t estr[2] = {1, 1};
  CUresult cr = encodeTiled()(&map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, p.lv[0].ptr, dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return cudaErrorInvalidValue;
  const uint64_t regions = uint64_t(tp.st.regionsX) * tp.st.regionsY;
  const uint32_t grid = uint32_t(std::min<uint64_t>(regions, uint64_t(info->sms)));
  void* args[] = {&map, &tp};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = kSmemBytes;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;  // see griddepcontrol in the kernel
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelExC(&cfg, tmaKernel(p.sharedFmt), args);
  if (e != cudaSuccess) return e;
  ++*launches;
  return cudaGetLastError();
}

// Device scratch for nvproPyramidGenerateNoAlloc: the shared error flag and
// the per-launch counters of a chain (see kStaticScratchWords).  It is a
// file-scope __device__ array, so every GPU that loads the library holds these
// 1 KiB until the process exits, and no call allocates.
static __device__ __align__(256) uint32_t g_staticScratch[kStaticScratchWords];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);

CtxGetCurrentFn ctxGetCurrent() {
  static CtxGetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return CtxGetCurrentFn(nullptr);
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

cudaError_t staticScratch(uint32_t** ptr) {
  struct Entry {
    CUcontext ctx;
    uint32_t* addr;
  };
  static Entry entries[64] = {};
  static std::mutex mu;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  CtxGetCurrentFn getCtx = ctxGetCurrent();
  CUcontext ctx = nullptr;
  if (getCtx && getCtx(&ctx) != CUDA_SUCCESS) ctx = nullptr;
  std::lock_guard<std::mutex> lock(mu);
  Entry& d = entries[dev];
  // A context that is not the one of the cached address (none yet, or the
  // device was reset and its context made anew, which may load the module at
  // another address) gets a fresh look-up.
  if (!d.addr || !ctx || ctx != d.ctx) {
    // In host code the array's name is a host-side stand-in; its device
    // address comes from the runtime, with the device current.
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_staticScratch);
    if (e != cudaSuccess) return e;
    if (getCtx && getCtx(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    d.addr = static_cast<uint32_t*>(p);
    d.ctx = ctx;
  }
  *ptr = d.addr;
  return cudaSuccess;
}

cudaError_t launchDebugMbarTimeout(uint32_t* errorFlag, cudaStream_t stream) {
  debugMbarTimeoutKernel<<<1, 32, 0, stream>>>(errorFlag);
  return cudaGetLastError();
}

cudaError_t launchDebugEncode(const float* x, uint8_t* fast, uint8_t* exact, uint64_t n, uint32_t alpha,
                              cudaStream_t stream) {
  DeviceInfo* info = nullptr;
  cudaError_t e = deviceInfo(&info);
  if (e != cudaSuccess) return e;
  debugEncodeKernel<<<info->sms * 2, 256, kDebugSmemBytes, stream>>>(x, fast, exact, n, alpha);
  return cudaGetLastError();
}

}  // namespace nvpyr
