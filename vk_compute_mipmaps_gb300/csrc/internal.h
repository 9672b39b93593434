// internal.h -- host-side types shared between the C ABI (api.cpp) and the
// kernel translation units.  Not part of the public interface.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nvpro_pyramid_rules.h"

namespace nvpyr {

using nvpro_pyramid::fastVerticalFirst;
using nvpro_pyramid::kernelSize;
using nvpro_pyramid::sharedHandoffLevel;

constexpr uint32_t kMaxDispatchLevels = 6;  // fast pipeline: 1..6 levels (nvpro_pyramid.glsl:221-225)
// Dispatches whose input level has at most this many texels run on the
// small-dispatch engine (small_engine.cuh), up to kMaxSmallDispatches per launch.
constexpr uint32_t kSmallMaxTexels = 64 * 64;
constexpr uint32_t kMaxSmallDispatches = 16;

enum Preset : uint32_t { kSrgba8 = 1, kRgba32f = 2, kRgba16f = 3 };

// Shared-memory formats of the sRGBA8 preset (srgba8_mipmap_preamble.glsl:60-108).
enum SharedFormat : uint32_t { kSharedFp32 = 0, kSharedSrgb = 1, kSharedF16 = 2 };

inline uint32_t presetBytes(uint32_t preset) {
  return preset == kSrgba8 ? 4u : preset == kRgba32f ? 16u : preset == kRgba16f ? 8u : 0u;
}

// One level of an image as a kernel sees it.
struct LevelView {
  uint8_t* ptr;
  uint64_t pitch;  // bytes between rows
  uint32_t w, h;
};

// Everything one recorded dispatch needs: the reference's push constant
// decoded, the workgroup coverage, and levels L..L+n.
struct DispatchParams {
  uint32_t preset;
  uint32_t isFast;
  uint32_t inputLevel;  // L
  uint32_t levelCount;  // n
  uint64_t groups;      // reference workgroups covered (gx if gy, gz > 0, else 0)
  // Format of the values handed through the reference's shared memory
  // (sRGBA8 only): kSharedFp32, kSharedSrgb or kSharedF16.
  uint32_t sharedFmt;
  uint32_t isBlit;  // a linear blit of one level (isFast 0, levelCount 1)
  LevelView lv[kMaxDispatchLevels + 1];
  // Strided batches (portable kernels only): `batch` images, image i's level
  // L+k at lv[k].ptr + i * imageStride[k].
  uint32_t batch = 1;
  uint64_t imageStride[kMaxDispatchLevels + 1] = {};
  // Custom pipelines (nvproPyramidCreateCustomPipeline): the launcher
  // (nvpro_pyramid_launcher_t) and its user data; null for the presets.
  void* launcher = nullptr;
  void* userData = nullptr;
};

// Scratch counter slots.
constexpr uint32_t kCounterLastCta = 0;
constexpr uint32_t kCounterError = 1;
constexpr uint32_t kCounterBarrier = 2;     // general chain: CTAs arrived at the barrier
constexpr uint32_t kCounterBarrierGen = 3;  // general chain: barrier generation
constexpr uint32_t kCounterExit = 4;        // general chain: CTAs that have exited (repairs the barrier count)

// Device scratch of a launch: counter words owned by a command object
// (allocated at creation) or a slice of the fixed no-allocation array.
struct Scratch {
  uint32_t* counters;     // zero-initialised, self-resetting
  uint32_t counterCount;
  // Where a bounded wait that gives up records it; null: counters + kCounterError.
  uint32_t* errorFlag = nullptr;
  uint32_t* error() const { return errorFlag ? errorFlag : counters + kCounterError; }
};

// Workgroups that cover every tile of a fast dispatch (nvpro_pyramid::fastGroupsNeeded).
inline uint64_t fastGroupsNeeded(const DispatchParams& p) {
  return nvpro_pyramid::fastGroupsNeeded(p.lv[0].w, p.lv[0].h, p.levelCount);
}

// True if the dispatch's workgroups cover every texel it can write (the
// default dispatchers always do; a caller's dispatcher may dispatch fewer).
inline bool dispatchCoversAll(const DispatchParams& p) {
  if (p.isBlit) return false;
  if (p.isFast) return p.groups >= fastGroupsNeeded(p);
  const LevelView &l1 = p.lv[1], &l2 = p.lv[2];
  if (p.levelCount == 1) return p.groups * 128u >= uint64_t(l1.w) * l1.h;
  return p.groups >= uint64_t((l2.w + 7) / 8) * ((l2.h + 7) / 8);
}

// Kernel families.  Each returns cudaSuccess or the launch error, and adds the
// number of kernels it launched to *launches.
cudaError_t launchPortable(const DispatchParams& p, cudaStream_t stream, uint32_t* launches);
// True if the TMA fast-pipeline kernel can run this dispatch (layout, alignment).
bool tmaFastSupported(const DispatchParams& p);
// The TMA kernel runs dispatch p, then (its last CTA) the tailCount small
// dispatches after it (smallDispatchSupported each, consecutive levels).
// debugFailCta (test support): that CTA gives up at once, as after a wait
// that ran out; ~0u = none.
cudaError_t launchTmaFast(const DispatchParams& p, const DispatchParams* tail, uint32_t tailCount,
                          cudaStream_t stream, const Scratch& scratch, uint32_t* launches,
                          uint32_t debugFailCta = ~0u);
// Test support: the fast sRGB encoder and the exact threshold count, per float.
cudaError_t launchDebugEncode(const float* x, uint8_t* fast, uint8_t* exact, uint64_t n, uint32_t alpha,
                              cudaStream_t stream);

// Adjoint of the linear float pyramids (kernels_adjoint.cu).  Gradient
// levels are RGBA FP32 (type 0) or RGBA FP16 (type 1); a null level reads as 0.
struct AdjointChainParams {
  uint32_t n;  // levels of the fast dispatch
  uint32_t w, h;  // size of level L
  uint32_t gType;
  const uint8_t* g[kMaxDispatchLevels];  // upstream gradient of levels L..L+n-1
  uint64_t gPitch[kMaxDispatchLevels];
  const uint8_t* top;  // h of level L+n
  uint64_t topPitch;
  uint32_t topType;
  uint32_t outType;
  uint8_t* out;  // h of level L
  uint64_t outPitch;
  // strided batches: image z at + z * stride (grid z = image)
  uint32_t batch;
  uint64_t gImage[kMaxDispatchLevels];
  uint64_t topImage, outImage;
};
struct AdjointLevelParams {
  uint32_t fw, fh, cw, ch;  // fine level k, coarse level k+1
  const uint8_t* g;         // upstream gradient of level k
  uint64_t gPitch;
  uint32_t gType;
  const uint8_t* hc;  // h of level k+1
  uint64_t hcPitch;
  uint32_t hcType;
  uint8_t* out;  // h of level k
  uint64_t outPitch;
  uint32_t outType;
  uint32_t batch;  // strided batches: image z at + z * stride (grid z = image)
  uint64_t gImage, hcImage, outImage;
};
// The general pipeline for sRGBA8 as streaming column strips
// (kernels_general.cu): dispatches of 1 or 2 levels whose input level is at
// least 2x2 (and level L+1 too, for 2 levels) with full workgroup coverage.
// A run of up to generalMaxStages() such dispatches is one cooperative launch
// with grid barriers between them, followed by up to kMaxSmallDispatches small
// dispatches that the last CTA runs; with no strip stages the launch is one
// CTA running small dispatches only.  A launch of more than one part uses
// scratch words kCounterError (or scratch.errorFlag), kCounterBarrier,
// kCounterBarrierGen and kCounterExit.
bool generalFastSupported(const DispatchParams& p);
uint32_t generalMaxStages();
cudaError_t launchGeneralChain(const DispatchParams* p, uint32_t count, const DispatchParams* small,
                               uint32_t smallCount, cudaStream_t stream, const Scratch& scratch, uint32_t* launches);
// True if the small-dispatch engine runs p: sRGBA8, a dispatch (not a blit)
// covering all its texels, one image, sizes within smallDispatchFits.
bool smallDispatchSupported(const DispatchParams& p);

// Premultiplied-alpha staging of sRGBA8 texels (kernels_stage.cu); src may equal dst.
cudaError_t launchPremultiply(const uint8_t* src, uint64_t srcPitch, uint8_t* dst, uint64_t dstPitch, uint32_t width,
                              uint32_t height, cudaStream_t stream);

// Speed-of-light probe (kernels_stage.cu): the traffic of a chain, no filtering.
cudaError_t launchProbe(const uint8_t* const* levels, const uint64_t* pitches, uint32_t width, uint32_t height,
                        uint32_t levelCount, cudaStream_t stream);

// Test support for failure detection: a bounded wait that runs out (an
// mbarrier phase nothing completes; a grid barrier nothing releases) and
// sets the error flag of `scratch` (scratch.error()) / errorFlag.
cudaError_t launchDebugMbarTimeout(uint32_t* errorFlag, cudaStream_t stream);
cudaError_t launchDebugGridBarrierTimeout(const Scratch& scratch, cudaStream_t stream);

cudaError_t launchAdjointChain(const AdjointChainParams& p, cudaStream_t stream);
cudaError_t launchAdjointLevel(const AdjointLevelParams& p, cudaStream_t stream);

// Words a launch uses: TMA fast kernel (last-CTA counter, error flag) and a
// general chain of two or more stages (error flag, barrier count, generation,
// exit count; slot 0 unused).
constexpr uint32_t kTmaScratchWords = kCounterError + 1;
constexpr uint32_t kGeneralScratchWords = kCounterExit + 1;

// The fixed device scratch of nvproPyramidGenerateNoAlloc: kStaticScratchWords
// words in a file-scope __device__ array.  Word kStaticErrorWord is the error
// flag of every launch of that path (kept until nvproPyramidNoAllocDeviceStatus
// reads and clears it); the words after it are the per-launch counters, which
// each call clears.  A chain has at most NVPRO_PYRAMID_MAX_LEVELS - 1
// dispatches, each launch covers at least one, and no launch needs more than
// kGeneralScratchWords words, so every chain fits.  Returns the array's device
// address for the current device and context, looked up (cudaGetSymbolAddress)
// on first use there.
constexpr uint32_t kStaticScratchWords = 256;
constexpr uint32_t kStaticErrorWord = 0;
static_assert(kStaticScratchWords >= 1 + 31 * kGeneralScratchWords, "a chain's launches must fit the fixed array");
cudaError_t staticScratch(uint32_t** ptr);

// Set the calling thread's nvproPyramidLastError text.
void setLastError(const char* text);

}  // namespace nvpyr
