// kernels_general.cu -- the sRGBA8 general pipeline (nvpro_pyramid.glsl:536-885)
// for GB300: one or two levels of the energy-conserving 2/3-tap kernel per
// dispatch, as warp-wide column strips that stream down the image, and a run
// of consecutive general dispatches in one persistent launch.
//
// The strips themselves are described in general_strip.cuh.
//
// Chains.  The dispatches of a run are the stages of one cooperative launch
// (all CTAs resident): the sRGB tables are filled once, and a grid barrier
// separates the stages, as the reference's pipeline barriers separate its
// dispatches (nvpro_pyramid_dispatch.hpp:150-160).  The barrier's wait is
// bounded: after kWaitLimit polls it sets the error flag and the kernel
// returns.  The small dispatches after the run (input levels of at most
// kSmallMaxTexels texels, of either pipeline) are the tail of the launch: the
// last CTA to finish the strips runs them with the small-dispatch engine
// (small_engine.cuh); a chain that starts small is one CTA running the engine.
// A launch without grid barriers (one strip stage or none) is an ordinary
// programmatic dependent launch, whose table fill overlaps the previous kernel.
#include <mutex>

#include "general_strip.cuh"
#include "small_engine.cuh"

namespace nvpyr {
namespace {

constexpr uint32_t kWarps = 12;
constexpr uint32_t kThreads = 32 * kWarps;
constexpr uint32_t kCtasPerSm = 1;
constexpr uint32_t kMaxStages = 16;
// the aligned tables, then the small-dispatch engine's buffers
constexpr uint32_t kSmemBytes = kAlignedLutSmemBytes + kSmallArenaBytes;
static_assert(kCtasPerSm * (kSmemBytes + 1024u) <= 228u * 1024u, "the CTAs of an SM must fit");

struct ChainParams {
  Stage st[kMaxStages];  // strip stages, all CTAs
  uint32_t stageCount;
  SmallDispatch tail[kMaxSmallDispatches];  // then small dispatches, one CTA
  uint32_t tailCount;
  uint32_t* barrierCount;  // CTAs arrived at the current barrier (self-resetting)
  uint32_t* barrierGen;    // barrier generation (only ever incremented)
  uint32_t* errorFlag;     // set to 1 if a bounded wait gave up
  uint32_t* exitCount;     // CTAs that have left (self-resetting; see exitArrive)
};

__device__ __forceinline__ bool gridBarrier(const ChainParams& p, uint32_t& gen, uint32_t* okFlag) {
  return gridBarrierWait(p.barrierCount, p.barrierGen, p.errorFlag, gen, okFlag);
}

template <uint32_t SF>
__device__ __forceinline__ void runStage(const Stage& st, uint32_t lane, uint32_t warpId, uint32_t warps, const Lut& L) {
  const uint32_t units = st.tilesX * st.bands;
  for (uint32_t u = warpId; u < units; u += warps) strip<SF>(st, u % st.tilesX, u / st.tilesX, lane, L);
}

// Every CTA of a multi-stage launch arrives here once on its way out.  The
// last one resets the barrier count: after a bounded wait gave up, CTAs leave
// at different barriers and the count can be left partial; the reset puts it
// back to zero for the next launch (no CTA uses it any more).
__device__ __forceinline__ void exitArrive(const ChainParams& p) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(p.exitCount, 1u) == gridDim.x - 1) {
      atomicExch(p.barrierCount, 0u);
      atomicExch(p.exitCount, 0u);
      __threadfence();
    }
  }
}

// SF: the general pipeline's shared format (one per launch).
template <uint32_t SF>
__global__ void __launch_bounds__(kThreads, kCtasPerSm) generalChainKernel(const __grid_constant__ ChainParams p) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint32_t okFlag;
  const Lut L = fillAlignedLut(smem, threadIdx.x, kThreads);
  // A launch without grid barriers is a programmatic dependent launch: the
  // table fill above may overlap the end of the previous kernel on the stream;
  // the first global access waits here for it to complete.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const bool multi = p.stageCount + (p.tailCount ? 1 : 0) > 1;  // uses the scratch counters
  uint32_t gen = 0;
  if (threadIdx.x == 0 && p.stageCount > 1) gen = ldAcquire(p.barrierGen);  // before this CTA's first arrival
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warpId = blockIdx.x * kWarps + (threadIdx.x >> 5), warps = gridDim.x * kWarps;
  bool ok = true;
#pragma unroll 1
  for (uint32_t s = 0; s < p.stageCount; ++s) {
    runStage<SF>(p.st[s], lane, warpId, warps, L);
    if (s + 1 < p.stageCount && !gridBarrier(p, gen, &okFlag)) {
      ok = false;
      break;
    }
  }
  // the small dispatches: by the last CTA to finish the strips (a hand-off
  // without waiting), or by the only CTA
  if (ok && p.tailCount && (p.stageCount == 0 || lastCtaArrives(p.barrierCount, &okFlag)))
    runSmallDispatches(p.tail, p.tailCount, smem + kAlignedLutSmemBytes, AlignedLutCodec{L}, threadIdx.x,
                       kThreads);
  if (multi) exitArrive(p);
}

// Test support for failure detection: one CTA arrives at the chain kernels'
// bounded grid barrier with the arrival count raised by two, as if two CTAs
// had arrived that will never release it; the wait gives up after its limit
// and sets the error flag.  The counters are left for the host to reset.
__global__ void debugGridBarrierTimeoutKernel(uint32_t* count, uint32_t* genWord, uint32_t* errorFlag) {
  __shared__ uint32_t okFlag;
  uint32_t gen = 0;
  if (threadIdx.x == 0) {
    atomicAdd(count, 2u);
    gen = ldAcquire(genWord);
  }
  gridBarrierWait(count, genWord, errorFlag, gen, &okFlag);
}

struct DeviceState {
  int sms = 0;
  int ctasPerSm = 0;
};

const void* chainKernel(uint32_t sharedFmt) {
  return sharedFmt == kSharedSrgb  ? reinterpret_cast<const void*>(generalChainKernel<kSharedSrgb>)
         : sharedFmt == kSharedF16 ? reinterpret_cast<const void*>(generalChainKernel<kSharedF16>)
                                   : reinterpret_cast<const void*>(generalChainKernel<kSharedFp32>);
}

cudaError_t deviceState(int* sms, int* ctasPerSm) {
  static DeviceState states[64];
  static std::mutex mu;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  DeviceState& d = states[dev];
  if (d.sms == 0) {
    int coop = 0;
    e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (e != cudaSuccess) return e;
    if (!coop) return cudaErrorNotSupported;
    for (const uint32_t fmt : {kSharedFp32, kSharedSrgb, kSharedF16}) {
      e = cudaFuncSetAttribute(chainKernel(fmt), cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemBytes));
      if (e != cudaSuccess) return e;
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.ctasPerSm, generalChainKernel<kSharedFp32>,
                                                      kThreads, kSmemBytes);
    if (e != cudaSuccess) return e;
    if (d.ctasPerSm < 1) return cudaErrorInvalidConfiguration;
    e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  *sms = d.sms;
  *ctasPerSm = d.ctasPerSm;
  return cudaSuccess;
}

void makeStage(const DispatchParams& p, uint64_t warpsResident, Stage* g) {
  stageGeometry(p, g);
  // Bands: about one strip per resident warp (a band's warp walks its rows
  // serially).
  const uint32_t lastH = g->variant < 16 ? g->h2 : g->h1;
  setStageBand(g, uint32_t(std::min<uint64_t>((uint64_t(g->tilesX) * lastH + warpsResident - 1) / warpsResident,
                                               lastH)));
}

}  // namespace

bool generalFastSupported(const DispatchParams& p) {
  if (p.preset != kSrgba8 || p.isFast || p.isBlit || (p.levelCount != 1 && p.levelCount != 2)) return false;
  const LevelView &l0 = p.lv[0], &l1 = p.lv[1];
  if (l0.w < 2 || l0.h < 2) return false;  // one-tap axes: the small-dispatch engine or the portable kernels
  if (p.levelCount == 2 && (l1.w < 2 || l1.h < 2)) return false;
  return dispatchCoversAll(p);
}

bool smallDispatchSupported(const DispatchParams& p) {
  return p.preset == kSrgba8 && !p.isBlit && p.batch <= 1 && p.levelCount >= 1 &&
         p.levelCount <= kMaxDispatchLevels && dispatchCoversAll(p) && smallDispatchFits(p);
}

uint32_t generalMaxStages() { return kMaxStages; }

cudaError_t launchDebugGridBarrierTimeout(const Scratch& scratch, cudaStream_t stream) {
  if (scratch.counterCount < kGeneralScratchWords) return cudaErrorInvalidValue;
  debugGridBarrierTimeoutKernel<<<1, 32, 0, stream>>>(scratch.counters + kCounterBarrier,
                                                       scratch.counters + kCounterBarrierGen, scratch.error());
  return cudaGetLastError();
}

cudaError_t launchGeneralChain(const DispatchParams* p, uint32_t count, const DispatchParams* small,
                               uint32_t smallCount, cudaStream_t stream, const Scratch& scratch, uint32_t* launches) {
  const bool multi = count + (smallCount ? 1 : 0) > 1;
  if (count + smallCount == 0 || count > kMaxStages || smallCount > kMaxSmallDispatches ||
      (multi && scratch.counterCount < kGeneralScratchWords))
    return cudaErrorInvalidValue;
  for (uint32_t i = 1; i < count; ++i)
    if (p[i].sharedFmt != p[0].sharedFmt) return cudaErrorInvalidValue;  // one shared format per launch
  int sms = 0, ctasPerSm = 0;
  cudaError_t e = deviceState(&sms, &ctasPerSm);
  if (e != cudaSuccess) return e;
  const uint32_t ctas = uint32_t(std::min(sms * ctasPerSm, sms * int(kCtasPerSm)));
  ChainParams cp{};
  cp.stageCount = count;
  uint64_t maxUnits = 0;
  for (uint32_t i = 0; i < count; ++i) {
    makeStage(p[i], uint64_t(ctas) * kWarps, &cp.st[i]);
    maxUnits = std::max<uint64_t>(maxUnits, uint64_t(cp.st[i].tilesX) * cp.st[i].bands);
  }
  cp.tailCount = smallCount;
  for (uint32_t i = 0; i < smallCount; ++i) makeSmallDispatch(small[i], &cp.tail[i]);
  if (multi) {
    cp.barrierCount = scratch.counters + kCounterBarrier;
    cp.barrierGen = scratch.counters + kCounterBarrierGen;
    cp.errorFlag = scratch.error();
    cp.exitCount = scratch.counters + kCounterExit;
  }
  // a single stage needs no more CTAs than its strips fill; small dispatches only: one
  uint32_t grid = count > 1 ? ctas : uint32_t(std::min<uint64_t>((maxUnits + kWarps - 1) / kWarps, ctas));
  if (count == 0) grid = 1;
  void* args[] = {&cp};
  const uint32_t fmt = count ? p[0].sharedFmt : kSharedFp32;  // the engine applies each dispatch's own format
  if (count > 1) {  // grid barriers: every CTA must be resident
    e = cudaLaunchCooperativeKernel(chainKernel(fmt), dim3(grid), dim3(kThreads), args, kSmemBytes, stream);
  } else {  // no CTA waits for another: an ordinary launch, programmatic dependent on the previous kernel
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = kSmemBytes;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelExC(&cfg, chainKernel(fmt), args);
  }
  if (e != cudaSuccess) return e;
  ++*launches;
  return cudaSuccess;
}

}  // namespace nvpyr
