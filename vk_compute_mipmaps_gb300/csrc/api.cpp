// api.cpp -- the C ABI of include/nvpro_pyramid_cuda.h: pipelines, images,
// the command recorder and the level scheduler (nvproCmdPyramidDispatch).
//
// Recording mirrors nvpro_pyramid_dispatch.hpp call for call.  At
// nvproPyramidEndCmd the recorded dispatches are lowered to kernel launches
// on the command's stream; stream order takes the place of the reference's
// compute->compute barriers.  Small trailing dispatches may be folded into
// the tail of the preceding kernel (NVPRO_PYRAMID_CMD_NO_FUSION disables it);
// the bytes written are the same either way.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/nvpro_pyramid_cuda.h"
#include "batch.h"
#include "internal.h"

using namespace nvpyr;

namespace {

thread_local std::string t_lastError;

NvproPyramidResult fail(NvproPyramidResult r, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_lastError = buf;
  return r;
}

constexpr uint32_t kPipelineMagic = 0x50595250u;  // "PRYP"
constexpr uint32_t kCmdMagic = 0x434D4450u;       // "PDMC"

uint32_t levelDim(uint32_t base, uint32_t k) {
  const uint32_t d = k >= 32 ? 0u : base >> k;
  return d ? d : 1u;
}

}  // namespace

struct NvproPyramidPipeline_T {
  uint32_t magic;
  uint32_t preset;  // NVPRO_PYRAMID_PRESET_* or NVPRO_PYRAMID_PRESET_CUSTOM
  uint32_t isFast;
  uint32_t configBits;
  uint32_t texelBytes;
  nvpro_pyramid_launcher_t launcher;  // custom pipelines
  void* userData;
};

struct Record {
  NvproPyramidDispatchRecord info;
  NvproPyramidImage image;
  uint32_t texelBytes;  // of the bound pipeline
  nvpro_pyramid_launcher_t launcher;
  void* userData;
};

struct NvproPyramidCmd_T {
  uint32_t magic;
  uint32_t flags;
  cudaStream_t stream = nullptr;
  bool recording = false;
  bool imageBound = false;
  NvproPyramidImage image{};
  NvproPyramidPipeline pipeline = nullptr;
  bool pipelineBoundSinceDispatch = false;
  bool barrierSinceDispatch = false;
  uint32_t pushConstant = 0;
  bool pushConstantSet = false;
  NvproPyramidResult error = NVPRO_PYRAMID_SUCCESS;
  std::string errorText;
  std::vector<Record> records;
  uint32_t launches = 0;
  Scratch scratch{nullptr, 0};
  // set by nvproPyramidGenerateStrided for the duration of one EndCmd
  uint32_t batch = 1;
  uint64_t imageStrides[NVPRO_PYRAMID_MAX_LEVELS] = {};
  // nvproPyramidDebugForceWaitTimeout(cmd, 2): CTA 0 of the next TMA launch gives up at once
  bool debugFailNextTma = false;
};

namespace {

bool validCmd(NvproPyramidCmd cmd) { return cmd && cmd->magic == kCmdMagic; }
bool validPipeline(NvproPyramidPipeline p) { return p && p->magic == kPipelineMagic; }

// Record a sticky error on the command (reported again by nvproPyramidEndCmd).
NvproPyramidResult cmdFail(NvproPyramidCmd cmd, NvproPyramidResult r, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_lastError = buf;
  if (validCmd(cmd) && cmd->error == NVPRO_PYRAMID_SUCCESS) {
    cmd->error = r;
    cmd->errorText = buf;
  }
  return r;
}

// Build kernel parameters for a record; checks the image against the dispatch.
NvproPyramidResult makeParams(const Record& rec, DispatchParams* out) {
  const NvproPyramidImage& img = rec.image;
  const uint32_t L = rec.info.pushConstant >> NVPRO_PYRAMID_INPUT_LEVEL_SHIFT;
  const uint32_t n = rec.info.pushConstant & 31u;
  const uint32_t bpp = rec.texelBytes;
  if (n == 0) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "dispatch with level count 0");
  if (rec.info.isBlit && n != 1) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "a blit fills one level");
  if (rec.info.isFastPipeline ? n > kMaxDispatchLevels : n > 2)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "%s pipeline cannot fill %u levels in one dispatch",
                rec.info.isFastPipeline ? "fast" : "general", n);
  if (uint64_t(L) + n >= img.levelCount)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "dispatch writes level %u but the image has %u levels",
                L + n, img.levelCount);
  std::memset(out, 0, sizeof *out);
  out->batch = 1;  // one image unless a strided call says otherwise
  out->preset = rec.info.preset;
  out->isFast = rec.info.isFastPipeline;
  out->isBlit = rec.info.isBlit;
  out->inputLevel = L;
  out->levelCount = n;
  out->groups = (rec.info.groupCountY == 0 || rec.info.groupCountZ == 0) ? 0 : rec.info.groupCountX;
  out->launcher = reinterpret_cast<void*>(rec.launcher);
  out->userData = rec.userData;
  out->sharedFmt = (rec.info.configBits & NVPRO_PYRAMID_CONFIG_SRGB_SHARED)  ? kSharedSrgb
                   : (rec.info.configBits & NVPRO_PYRAMID_CONFIG_F16_SHARED) ? kSharedF16
                                                                             : kSharedFp32;
  const uint32_t align = std::min(16u, bpp & (0u - bpp));  // largest power of two dividing bpp, at most 16
  for (uint32_t k = 0; k <= n; ++k) {
    const uint32_t lvl = L + k;
    LevelView& v = out->lv[k];
    v.w = levelDim(img.width, lvl);
    v.h = levelDim(img.height, lvl);
    v.ptr = static_cast<uint8_t*>(img.levels[lvl]);
    v.pitch = img.rowPitchBytes[lvl] ? img.rowPitchBytes[lvl] : uint64_t(v.w) * bpp;
    if (!v.ptr) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "level %u has no device pointer", lvl);
    if (v.pitch < uint64_t(v.w) * bpp)
      return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "level %u row pitch %llu < %u texels", lvl,
                  (unsigned long long)v.pitch, v.w);
    if ((reinterpret_cast<uintptr_t>(v.ptr) % align) || (v.pitch % align))
      return fail(NVPRO_PYRAMID_ERROR_UNSUPPORTED, "level %u pointer/pitch not %u-byte aligned", lvl, align);
  }
  return NVPRO_PYRAMID_SUCCESS;
}

// How recorded dispatches become kernel launches.
enum LaunchKind : uint32_t {
  kLaunchTma = 0,      // the TMA fast kernel: dispatch `first`, then `small` small dispatches in its tail
  kLaunchGeneral = 1,  // the general chain: `big` strip stages from `first`, then `small` small dispatches
  kLaunchSmall = 2,    // one CTA: `small` small dispatches from `first`
  kLaunchPortable = 3,  // the portable kernels: dispatch `first`
  kLaunchCustom = 4     // a custom pipeline's launcher: dispatch `first`
};
struct LaunchPlan {
  uint32_t kind, first, big, small;
  // scratch words the launch needs (the counters of launches of several parts)
  uint32_t words() const {
    if (kind == kLaunchTma) return small ? kTmaScratchWords : 0;
    if (kind == kLaunchGeneral) return big + (small ? 1 : 0) > 1 ? kGeneralScratchWords : 0;
    return 0;
  }
};

// `next` continues the level chain of `prev` (its input is prev's last level).
bool continues(const DispatchParams& prev, const DispatchParams& next) {
  const LevelView& out = prev.lv[prev.levelCount];
  return next.inputLevel == prev.inputLevel + prev.levelCount && next.lv[0].ptr == out.ptr &&
         next.lv[0].pitch == out.pitch;
}

// Lower n dispatches to launches.  Small dispatches (smallDispatchSupported)
// after a launch's large work run in that launch's last CTA; a run that
// starts small is one single-CTA launch.  `fuse` false: one dispatch per
// launch; `portableOnly`: every dispatch on the portable kernels.
uint32_t planLaunches(const DispatchParams* p, uint32_t n, bool fuse, bool portableOnly, LaunchPlan* out) {
  uint32_t count = 0;
  // small dispatches continuing the chain from dispatch j on (at most `room`)
  auto smallRun = [&](uint32_t j, uint32_t room) {
    uint32_t k = j;
    while (fuse && k < n && k - j < room && smallDispatchSupported(p[k]) && (k == j || continues(p[k - 1], p[k])))
      ++k;
    return k - j;
  };
  for (uint32_t i = 0; i < n;) {
    LaunchPlan& l = out[count++];
    l = LaunchPlan{kLaunchPortable, i, 1, 0};
    if (p[i].launcher) {
      l.kind = kLaunchCustom;
      i += 1;
    } else if (portableOnly) {
      i += 1;
    } else if (smallDispatchSupported(p[i])) {
      l.kind = kLaunchSmall;
      l.big = 0;
      l.small = fuse ? smallRun(i, kMaxSmallDispatches) : 1;
      i += l.small;
    } else if (p[i].isFast && tmaFastSupported(p[i])) {
      l.kind = kLaunchTma;
      l.small = smallRun(i + 1, kMaxSmallDispatches);
      i += 1 + l.small;
    } else if (generalFastSupported(p[i])) {
      uint32_t j = i + 1;
      while (fuse && j < n && j - i < generalMaxStages() && generalFastSupported(p[j]) &&
             !smallDispatchSupported(p[j]) && p[j].sharedFmt == p[i].sharedFmt)
        ++j;
      l.kind = kLaunchGeneral;
      l.big = j - i;
      l.small = smallRun(j, kMaxSmallDispatches);
      i = j + l.small;
    } else {
      i += 1;
    }
  }
  return count;
}

// A dispatch of a custom pipeline through its launcher.
NvproPyramidResult launchCustom(const DispatchParams& p, cudaStream_t stream) {
  NvproPyramidDispatchDesc d{};
  d.isFastPipeline = p.isFast;
  d.inputLevel = p.inputLevel;
  d.levelCount = p.levelCount;
  d.imageCount = p.batch;
  d.groupCount = p.groups;
  for (uint32_t k = 0; k <= p.levelCount; ++k)
    d.levels[k] = NvproPyramidLevelDesc{p.lv[k].ptr, p.lv[k].pitch, p.lv[k].w, p.lv[k].h, p.imageStride[k]};
  const auto fn = reinterpret_cast<nvpro_pyramid_launcher_t>(p.launcher);
  const NvproPyramidResult r = fn(p.userData, reinterpret_cast<NvproPyramidStream>(stream), &d);
  return r == NVPRO_PYRAMID_SUCCESS ? r : fail(r, "custom pipeline launcher: %s", nvproPyramidResultString(r));
}

// Enqueue one planned launch with the given scratch.
cudaError_t runLaunch(const LaunchPlan& l, const DispatchParams* p, cudaStream_t s, const Scratch& scratch,
                      uint32_t* launches, uint32_t debugFailCta = ~0u) {
  const DispatchParams* d = p + l.first;
  switch (l.kind) {
    case kLaunchTma: return launchTmaFast(*d, l.small ? d + 1 : nullptr, l.small, s, scratch, launches, debugFailCta);
    case kLaunchGeneral: return launchGeneralChain(d, l.big, d + l.big, l.small, s, scratch, launches);
    case kLaunchSmall: return launchGeneralChain(d, 0, d, l.small, s, scratch, launches);
    default: return launchPortable(*d, s, launches);
  }
}

}  // namespace

extern "C" {

const char* nvproPyramidResultString(NvproPyramidResult r) {
  switch (r) {
    case NVPRO_PYRAMID_SUCCESS: return "success";
    case NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT: return "invalid argument";
    case NVPRO_PYRAMID_ERROR_INVALID_STATE: return "invalid state";
    case NVPRO_PYRAMID_ERROR_DISPATCHER: return "dispatcher contract violated";
    case NVPRO_PYRAMID_ERROR_UNSUPPORTED: return "unsupported";
    case NVPRO_PYRAMID_ERROR_CUDA: return "CUDA error";
    case NVPRO_PYRAMID_ERROR_OUT_OF_MEMORY: return "out of memory";
    case NVPRO_PYRAMID_ERROR_TIMEOUT: return "device wait timed out";
    case NVPRO_PYRAMID_ERROR_IO: return "file I/O failed";
  }
  return "unknown result";
}

const char* nvproPyramidLastError(void) { return t_lastError.c_str(); }

}  // extern "C"

void nvpyr::setLastError(const char* text) { t_lastError = text; }

extern "C" {

uint32_t nvproPyramidPresetTexelBytes(NvproPyramidPreset preset) { return presetBytes(uint32_t(preset)); }

NvproPyramidResult nvproPyramidCreatePipeline(NvproPyramidPreset preset, uint32_t isFastPipeline,
                                              NvproPyramidPipeline* pPipeline) {
  return nvproPyramidCreatePipelineEx(preset, isFastPipeline, 0, pPipeline);
}

NvproPyramidResult nvproPyramidCreatePipelineEx(NvproPyramidPreset preset, uint32_t isFastPipeline,
                                                uint32_t configBits, NvproPyramidPipeline* pPipeline) {
  if (!pPipeline) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "pPipeline is NULL");
  *pPipeline = nullptr;
  if (presetBytes(uint32_t(preset)) == 0)
    return fail(NVPRO_PYRAMID_ERROR_UNSUPPORTED, "unknown preset %d", int(preset));
  constexpr uint32_t kShared = NVPRO_PYRAMID_CONFIG_SRGB_SHARED | NVPRO_PYRAMID_CONFIG_F16_SHARED;
  if (configBits & ~(kShared | NVPRO_PYRAMID_CONFIG_NO_BILINEAR))
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "unknown configuration bits 0x%x", configBits);
  if ((configBits & kShared) == kShared)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "SRGB_SHARED and F16_SHARED are exclusive");
  if ((configBits & kShared) && preset != NVPRO_PYRAMID_PRESET_SRGBA8)
    return fail(NVPRO_PYRAMID_ERROR_UNSUPPORTED, "shared-memory formats exist for the sRGBA8 preset only");
  auto* p = new (std::nothrow) NvproPyramidPipeline_T{
      kPipelineMagic, uint32_t(preset), isFastPipeline ? 1u : 0u, configBits, presetBytes(uint32_t(preset)), nullptr,
      nullptr};
  if (!p) return fail(NVPRO_PYRAMID_ERROR_OUT_OF_MEMORY, "host allocation failed");
  *pPipeline = p;
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidCreateCustomPipeline(uint32_t isFastPipeline, uint32_t texelBytes,
                                                    nvpro_pyramid_launcher_t launcher, void* userData,
                                                    NvproPyramidPipeline* pPipeline) {
  if (!pPipeline) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "pPipeline is NULL");
  *pPipeline = nullptr;
  if (!launcher || texelBytes == 0 || texelBytes > 256)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "a custom pipeline needs a launcher and 1..256 bytes per texel");
  auto* p = new (std::nothrow) NvproPyramidPipeline_T{kPipelineMagic, NVPRO_PYRAMID_PRESET_CUSTOM,
                                                      isFastPipeline ? 1u : 0u, 0u, texelBytes, launcher, userData};
  if (!p) return fail(NVPRO_PYRAMID_ERROR_OUT_OF_MEMORY, "host allocation failed");
  *pPipeline = p;
  return NVPRO_PYRAMID_SUCCESS;
}

void nvproPyramidDestroyPipeline(NvproPyramidPipeline pipeline) {
  if (validPipeline(pipeline)) {
    pipeline->magic = 0;
    delete pipeline;
  }
}

uint32_t nvproPyramidFullLevelCount(uint32_t width, uint32_t height) {
  uint32_t m = 0;
  while (width != 0 || height != 0) {
    width >>= 1;
    height >>= 1;
    ++m;
  }
  return m;
}

NvproPyramidResult nvproPyramidPackedLayout(uint32_t width, uint32_t height, uint32_t levelCount,
                                            uint32_t bytesPerTexel, uint64_t* pOffsets) {
  if (!pOffsets) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "pOffsets is NULL");
  if (width == 0 || height == 0 || bytesPerTexel == 0)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "zero width, height or texel size");
  if (levelCount == 0 || levelCount > nvproPyramidFullLevelCount(width, height))
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "level count %u outside 1..%u", levelCount,
                nvproPyramidFullLevelCount(width, height));
  uint64_t off = 0;
  for (uint32_t k = 0; k < levelCount; ++k) {
    pOffsets[k] = off;
    off += uint64_t(levelDim(width, k)) * levelDim(height, k) * bytesPerTexel;
  }
  pOffsets[levelCount] = off;
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidImageInitPacked(NvproPyramidImage* pImage, void* base, uint32_t width,
                                               uint32_t height, uint32_t levelCount, uint32_t bytesPerTexel) {
  if (!pImage || !base) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "NULL image or base pointer");
  if (levelCount > NVPRO_PYRAMID_MAX_LEVELS)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "level count %u > %u", levelCount,
                NVPRO_PYRAMID_MAX_LEVELS);
  uint64_t off[NVPRO_PYRAMID_MAX_LEVELS + 1];
  NvproPyramidResult r = nvproPyramidPackedLayout(width, height, levelCount, bytesPerTexel, off);
  if (r != NVPRO_PYRAMID_SUCCESS) return r;
  std::memset(pImage, 0, sizeof *pImage);
  pImage->width = width;
  pImage->height = height;
  pImage->levelCount = levelCount;
  for (uint32_t k = 0; k < levelCount; ++k) {
    pImage->levels[k] = static_cast<uint8_t*>(base) + off[k];
    pImage->rowPitchBytes[k] = uint64_t(levelDim(width, k)) * bytesPerTexel;
  }
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidCreateCmd(uint32_t flags, NvproPyramidCmd* pCmd) {
  if (!pCmd) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "pCmd is NULL");
  *pCmd = nullptr;
  auto* c = new (std::nothrow) NvproPyramidCmd_T();
  if (!c) return fail(NVPRO_PYRAMID_ERROR_OUT_OF_MEMORY, "host allocation failed");
  c->magic = kCmdMagic;
  c->flags = flags;
  if (!(flags & NVPRO_PYRAMID_CMD_RECORD_ONLY)) {
    // Counters for in-kernel tail fusion: allocated once here, never while
    // recording or launching.
    const uint32_t count = 1024;
    void* ptr = nullptr;
    cudaError_t e = cudaMalloc(&ptr, count * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(ptr, 0, count * sizeof(uint32_t));
    if (e != cudaSuccess) {
      if (ptr) cudaFree(ptr);
      delete c;
      return fail(e == cudaErrorMemoryAllocation ? NVPRO_PYRAMID_ERROR_OUT_OF_MEMORY : NVPRO_PYRAMID_ERROR_CUDA,
                  "cudaMalloc of command counters failed: %s", cudaGetErrorString(e));
    }
    c->scratch.counters = static_cast<uint32_t*>(ptr);
    c->scratch.counterCount = count;
  }
  *pCmd = c;
  return NVPRO_PYRAMID_SUCCESS;
}

void nvproPyramidDestroyCmd(NvproPyramidCmd cmd) {
  if (!validCmd(cmd)) return;
  if (cmd->scratch.counters) cudaFree(cmd->scratch.counters);
  cmd->magic = 0;
  delete cmd;
}

NvproPyramidResult nvproPyramidBeginCmd(NvproPyramidCmd cmd, NvproPyramidStream stream) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  cmd->stream = reinterpret_cast<cudaStream_t>(stream);
  cmd->recording = true;
  cmd->imageBound = false;
  cmd->pipeline = nullptr;
  cmd->pipelineBoundSinceDispatch = false;
  cmd->barrierSinceDispatch = false;
  cmd->pushConstantSet = false;
  cmd->error = NVPRO_PYRAMID_SUCCESS;
  cmd->errorText.clear();
  cmd->records.clear();
  cmd->launches = 0;
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidCmdBindImage(NvproPyramidCmd cmd, const NvproPyramidImage* pImage) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (!cmd->recording) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "command is not recording");
  if (!pImage) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "pImage is NULL");
  if (pImage->width == 0 || pImage->height == 0)
    return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "image has zero width or height");
  if (pImage->levelCount == 0 || pImage->levelCount > NVPRO_PYRAMID_MAX_LEVELS ||
      pImage->levelCount > nvproPyramidFullLevelCount(pImage->width, pImage->height))
    return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "image level count %u invalid for %ux%u",
                   pImage->levelCount, pImage->width, pImage->height);
  cmd->image = *pImage;
  cmd->imageBound = true;
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidCmdBindPipeline(NvproPyramidCmd cmd, NvproPyramidPipeline pipeline) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (!cmd->recording) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "command is not recording");
  if (!validPipeline(pipeline)) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid pipeline");
  cmd->pipeline = pipeline;
  cmd->pipelineBoundSinceDispatch = true;
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidCmdPushConstants(NvproPyramidCmd cmd, const void* /*layout*/, uint32_t offset,
                                                uint32_t size, const void* pValues) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (!cmd->recording) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "command is not recording");
  if (!pValues || offset != 0 || size != 4)
    return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT,
                   "push constant must be 4 bytes at offset 0 (got %u at %u)", size, offset);
  std::memcpy(&cmd->pushConstant, pValues, 4);
  cmd->pushConstantSet = true;
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidCmdDispatch(NvproPyramidCmd cmd, uint32_t gx, uint32_t gy, uint32_t gz) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (!cmd->recording) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "command is not recording");
  if (!cmd->pipeline) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "dispatch with no bound pipeline");
  if (!cmd->imageBound) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "dispatch with no bound image");
  if (!cmd->pushConstantSet)
    return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "dispatch with no push constant set");
  Record r;
  std::memset(&r, 0, sizeof r);
  r.info.isFastPipeline = cmd->pipeline->isFast;
  r.info.preset = cmd->pipeline->preset;
  r.info.configBits = cmd->pipeline->configBits;
  r.info.pushConstant = cmd->pushConstant;
  r.info.groupCountX = gx;
  r.info.groupCountY = gy;
  r.info.groupCountZ = gz;
  r.info.pipelineBound = cmd->pipelineBoundSinceDispatch;
  r.info.barrierBefore = cmd->barrierSinceDispatch;
  r.image = cmd->image;
  r.texelBytes = cmd->pipeline->texelBytes;
  r.launcher = cmd->pipeline->launcher;
  r.userData = cmd->pipeline->userData;
  DispatchParams probe;
  NvproPyramidResult res = makeParams(r, &probe);
  if (res != NVPRO_PYRAMID_SUCCESS) return cmdFail(cmd, res, "%s", t_lastError.c_str());
  cmd->records.push_back(r);
  cmd->pipelineBoundSinceDispatch = false;
  cmd->barrierSinceDispatch = false;
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidCmdBlitLevel(NvproPyramidCmd cmd, uint32_t srcLevel) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (!cmd->recording) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "command is not recording");
  if (!cmd->pipeline) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "blit with no bound pipeline (preset)");
  if (!cmd->imageBound) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "blit with no bound image");
  if (srcLevel >= 31) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "source level %u", srcLevel);
  if (cmd->pipeline->launcher)
    return cmdFail(cmd, NVPRO_PYRAMID_ERROR_UNSUPPORTED, "blits exist for the built-in presets only");
  Record r;
  std::memset(&r, 0, sizeof r);
  r.info.isFastPipeline = 0;
  r.info.isBlit = 1;
  r.info.preset = cmd->pipeline->preset;
  r.info.pushConstant = srcLevel << NVPRO_PYRAMID_INPUT_LEVEL_SHIFT | 1u;
  r.info.groupCountX = r.info.groupCountY = r.info.groupCountZ = 1;
  r.info.pipelineBound = cmd->pipelineBoundSinceDispatch;
  r.info.barrierBefore = cmd->barrierSinceDispatch;
  r.image = cmd->image;
  r.texelBytes = cmd->pipeline->texelBytes;
  DispatchParams probe;
  NvproPyramidResult res = makeParams(r, &probe);
  if (res != NVPRO_PYRAMID_SUCCESS) return cmdFail(cmd, res, "%s", t_lastError.c_str());
  cmd->records.push_back(r);
  cmd->pipelineBoundSinceDispatch = false;
  cmd->barrierSinceDispatch = false;
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidCmdPipelineBarrier(NvproPyramidCmd cmd) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (!cmd->recording) return cmdFail(cmd, NVPRO_PYRAMID_ERROR_INVALID_STATE, "command is not recording");
  cmd->barrierSinceDispatch = true;
  return NVPRO_PYRAMID_SUCCESS;
}

uint32_t nvproPyramidCmdRecordCount(NvproPyramidCmd cmd) {
  return validCmd(cmd) ? uint32_t(cmd->records.size()) : 0u;
}

NvproPyramidResult nvproPyramidCmdGetRecords(NvproPyramidCmd cmd, NvproPyramidDispatchRecord* pRecords,
                                             uint32_t count) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (count > cmd->records.size() || (count && !pRecords))
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "asked for %u of %zu records", count, cmd->records.size());
  for (uint32_t i = 0; i < count; ++i) pRecords[i] = cmd->records[i].info;
  return NVPRO_PYRAMID_SUCCESS;
}

uint32_t nvproPyramidCmdLaunchCount(NvproPyramidCmd cmd) { return validCmd(cmd) ? cmd->launches : 0u; }

NvproPyramidResult nvproPyramidEndCmd(NvproPyramidCmd cmd) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (!cmd->recording) return fail(NVPRO_PYRAMID_ERROR_INVALID_STATE, "command is not recording");
  cmd->recording = false;
  cmd->launches = 0;
  if (cmd->error != NVPRO_PYRAMID_SUCCESS) {
    t_lastError = cmd->errorText;
    return cmd->error;
  }
  if (cmd->flags & NVPRO_PYRAMID_CMD_RECORD_ONLY) return NVPRO_PYRAMID_SUCCESS;

  std::vector<DispatchParams> params(cmd->records.size());
  for (size_t i = 0; i < cmd->records.size(); ++i) {
    NvproPyramidResult r = makeParams(cmd->records[i], &params[i]);
    if (r != NVPRO_PYRAMID_SUCCESS) return r;
    params[i].batch = cmd->batch;
    for (uint32_t k = 0; k <= params[i].levelCount; ++k)
      params[i].imageStride[k] = cmd->imageStrides[params[i].inputLevel + k];
  }
  const bool fuse = !(cmd->flags & NVPRO_PYRAMID_CMD_NO_FUSION);
  // strided batches run on the portable kernels (one launch per dispatch, grid z = image)
  const bool portableOnly = (cmd->flags & NVPRO_PYRAMID_CMD_PORTABLE_KERNELS) != 0 || cmd->batch > 1;
  std::vector<LaunchPlan> plan(params.size());
  plan.resize(planLaunches(params.data(), uint32_t(params.size()), fuse, portableOnly, plan.data()));
  for (const LaunchPlan& l : plan) {
    if (l.kind == kLaunchCustom) {
      const NvproPyramidResult r = launchCustom(params[l.first], cmd->stream);
      if (r != NVPRO_PYRAMID_SUCCESS) return r;
      ++cmd->launches;
      continue;
    }
    // the command's counters serve every launch: launches are stream-ordered
    // and each leaves its counters at zero
    const uint32_t failCta = (l.kind == kLaunchTma && cmd->debugFailNextTma) ? 0u : ~0u;
    if (l.kind == kLaunchTma) cmd->debugFailNextTma = false;
    const cudaError_t e = runLaunch(l, params.data(), cmd->stream, cmd->scratch, &cmd->launches, failCta);
    if (e != cudaSuccess)
      return fail(NVPRO_PYRAMID_ERROR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
  }
  return NVPRO_PYRAMID_SUCCESS;
}

// ---------------------------------------------------------------------------
// The dispatcher (nvpro_pyramid_dispatch.hpp:109-304).

uint32_t nvproPyramidFastDispatch(NvproPyramidCmd cmdBuf, const void* layout, uint32_t pushConstantOffset,
                                  NvproPyramidPipeline pipelineIfNeeded, const NvproPyramidState* state,
                                  uint32_t divisibilityRequirement, uint32_t maxLevels) {
  if (!state || divisibilityRequirement == 0 || divisibilityRequirement % 2 != 0 || maxLevels == 0 ||
      maxLevels > 6) {
    cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT,
            "fast dispatcher needs an even divisibility requirement and 1..6 levels");
    return 0;
  }
  if (state->currentX % divisibilityRequirement != 0 || state->currentY % divisibilityRequirement != 0) return 0;
  if (pipelineIfNeeded) nvproPyramidCmdBindPipeline(cmdBuf, pipelineIfNeeded);
  uint32_t x = state->currentX, y = state->currentY, levels = 0;
  while (x % 2 == 0 && y % 2 == 0 && levels < state->remainingLevels && levels < maxLevels) {
    x /= 2;
    y /= 2;
    ++levels;
  }
  const uint32_t pc = state->currentLevel << NVPRO_PYRAMID_INPUT_LEVEL_SHIFT | levels;
  nvproPyramidCmdPushConstants(cmdBuf, layout, pushConstantOffset, sizeof pc, &pc);
  // 4096 input samples per workgroup for 6 levels, else 1024 (:234-238);
  // the product wraps in 32 bits exactly as the reference computes it.
  const uint32_t shift = levels > 5 ? 12u : 10u, mask = levels > 5 ? 4095u : 1023u;
  const uint32_t samples = state->currentX * state->currentY;
  nvproPyramidCmdDispatch(cmdBuf, (samples + mask) >> shift, 1u, 1u);
  return levels;
}

uint32_t nvproPyramidDefaultFastDispatcher(NvproPyramidCmd cmdBuf, const void* layout, uint32_t pushConstantOffset,
                                           NvproPyramidPipeline pipelineIfNeeded, const NvproPyramidState* state) {
  return nvproPyramidFastDispatch(cmdBuf, layout, pushConstantOffset, pipelineIfNeeded, state, 4, 6);
}

uint32_t nvproPyramidDefaultGeneralDispatcher(NvproPyramidCmd cmdBuf, const void* layout,
                                              uint32_t pushConstantOffset, NvproPyramidPipeline pipelineIfNeeded,
                                              const NvproPyramidState* state) {
  // "py2_4_8_8" parameters (:254-258): 4 warps, 8x8 tiles, at most 2 levels.
  constexpr uint32_t kMaxLevels = 2, kThreads = 4 * 32, kTile = 8;
  if (!state) {
    cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "state is NULL");
    return 0;
  }
  if (pipelineIfNeeded) nvproPyramidCmdBindPipeline(cmdBuf, pipelineIfNeeded);
  const uint32_t levels = state->remainingLevels >= kMaxLevels ? kMaxLevels : state->remainingLevels;
  const uint32_t pc = state->currentLevel << NVPRO_PYRAMID_INPUT_LEVEL_SHIFT | levels;
  nvproPyramidCmdPushConstants(cmdBuf, layout, pushConstantOffset, sizeof pc, &pc);
  uint32_t dstW = state->currentX >> levels, dstH = state->currentY >> levels;
  dstW = dstW ? dstW : 1u;
  dstH = dstH ? dstH : 1u;
  if (levels == 1)
    nvproPyramidCmdDispatch(cmdBuf, (dstW * dstH + (kThreads - 1)) / kThreads, 1u, 1u);
  else
    nvproPyramidCmdDispatch(cmdBuf, ((dstW + kTile - 1) / kTile) * ((dstH + kTile - 1) / kTile), 1u, 1u);
  return levels;
}

uint32_t nvproPyramidBlitGeneralDispatcher(NvproPyramidCmd cmdBuf, const void* /*layout*/,
                                           uint32_t /*pushConstantOffset*/, NvproPyramidPipeline pipelineIfNeeded,
                                           const NvproPyramidState* state) {
  if (!state) {
    cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "state is NULL");
    return 0;
  }
  if (pipelineIfNeeded) nvproPyramidCmdBindPipeline(cmdBuf, pipelineIfNeeded);
  return nvproPyramidCmdBlitLevel(cmdBuf, state->currentLevel) == NVPRO_PYRAMID_SUCCESS ? 1u : 0u;
}

NvproPyramidResult nvproCmdPyramidDispatchEx(NvproPyramidCmd cmdBuf, NvproPyramidPipelines pipelines,
                                             uint32_t baseWidth, uint32_t baseHeight, uint32_t mipLevels,
                                             nvpro_pyramid_dispatcher_t generalDispatcher,
                                             nvpro_pyramid_dispatcher_t fastDispatcher) {
  if (!validCmd(cmdBuf)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (!cmdBuf->recording) return cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_INVALID_STATE, "command is not recording");
  if (!validPipeline(pipelines.generalPipeline))
    return cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "generalPipeline is mandatory");
  if (pipelines.fastPipeline && !validPipeline(pipelines.fastPipeline))
    return cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid fastPipeline");
  if (pipelines.pushConstantOffset != 0)
    return cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_UNSUPPORTED, "pushConstantOffset must be 0");
  if (!generalDispatcher || (pipelines.fastPipeline && !fastDispatcher))
    return cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "missing dispatcher callback");
  if (baseWidth == 0 || baseHeight == 0)
    return cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "zero base width or height");
  const uint32_t fullLevels = nvproPyramidFullLevelCount(baseWidth, baseHeight);
  if (mipLevels == 0) mipLevels = fullLevels;  // :122-132
  if (mipLevels > fullLevels)
    return cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "%u levels requested; %ux%u has at most %u",
                   mipLevels, baseWidth, baseHeight, fullLevels);
  // A single-level image needs no dispatch (the reference asserts here,
  // because its loop dispatches before testing remainingLevels).
  if (mipLevels == 1) return NVPRO_PYRAMID_SUCCESS;

  NvproPyramidState state{0u, mipLevels - 1u, baseWidth, baseHeight};
  NvproPyramidPipeline fastIfNeeded = pipelines.fastPipeline;
  NvproPyramidPipeline generalIfNeeded = pipelines.generalPipeline;
  while (true) {
    uint32_t done = 0;
    if (pipelines.fastPipeline)
      done = fastDispatcher(cmdBuf, pipelines.layout, pipelines.pushConstantOffset, fastIfNeeded, &state);
    if (done != 0) {
      fastIfNeeded = nullptr;
      generalIfNeeded = pipelines.generalPipeline;
    } else {
      done = generalDispatcher(cmdBuf, pipelines.layout, pipelines.pushConstantOffset, generalIfNeeded, &state);
      fastIfNeeded = pipelines.fastPipeline;
      generalIfNeeded = nullptr;
    }
    if (cmdBuf->error != NVPRO_PYRAMID_SUCCESS) return cmdBuf->error;
    if (done == 0 || done > state.remainingLevels)  // the reference's asserts (:169,:172)
      return cmdFail(cmdBuf, NVPRO_PYRAMID_ERROR_DISPATCHER,
                     "dispatcher filled %u levels with %u remaining at level %u", done, state.remainingLevels,
                     state.currentLevel);
    state.currentLevel += done;
    state.remainingLevels -= done;
    state.currentX = std::max(state.currentX >> done, 1u);
    state.currentY = std::max(state.currentY >> done, 1u);
    if (state.remainingLevels == 0) break;
    nvproPyramidCmdPipelineBarrier(cmdBuf);
  }
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproCmdPyramidDispatch(NvproPyramidCmd cmdBuf, NvproPyramidPipelines pipelines,
                                           uint32_t baseWidth, uint32_t baseHeight, uint32_t mipLevels) {
  return nvproCmdPyramidDispatchEx(cmdBuf, pipelines, baseWidth, baseHeight, mipLevels,
                                   nvproPyramidDefaultGeneralDispatcher, nvproPyramidDefaultFastDispatcher);
}

NvproPyramidResult nvproPyramidCmdDeviceStatus(NvproPyramidCmd cmd) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (!cmd->scratch.counters) return NVPRO_PYRAMID_SUCCESS;
  cudaError_t e = cudaStreamSynchronize(cmd->stream);
  uint32_t flag = 0;
  if (e == cudaSuccess)
    e = cudaMemcpy(&flag, cmd->scratch.counters + kCounterError, sizeof flag, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "device status: %s", cudaGetErrorString(e));
  if (flag) {
    // A kernel gave up waiting: clear the flag and the tail counter it may
    // have left behind.
    e = cudaMemset(cmd->scratch.counters, 0, cmd->scratch.counterCount * sizeof(uint32_t));
    if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "device status: %s", cudaGetErrorString(e));
    return fail(NVPRO_PYRAMID_ERROR_TIMEOUT, "a device-side wait gave up; outputs are incomplete");
  }
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidDebugForceWaitTimeout(NvproPyramidCmd cmd, uint32_t waitKind) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (!cmd->scratch.counters) return fail(NVPRO_PYRAMID_ERROR_INVALID_STATE, "command without device counters");
  cudaError_t e;
  if (waitKind == 0)
    e = launchDebugMbarTimeout(cmd->scratch.error(), cmd->stream);
  else if (waitKind == 1)
    e = launchDebugGridBarrierTimeout(cmd->scratch, cmd->stream);
  else if (waitKind == 2) {
    cmd->debugFailNextTma = true;
    e = cudaSuccess;
  } else
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "waitKind %u", waitKind);
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "launch failed: %s", cudaGetErrorString(e));
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidSpeedOfLightProbe(NvproPyramidStream stream, const NvproPyramidImage* pImage,
                                                uint32_t mipLevels) {
  if (!pImage) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "pImage is NULL");
  const uint32_t w = pImage->width, h = pImage->height;
  const uint32_t full = nvproPyramidFullLevelCount(w, h);
  if (mipLevels == 0) mipLevels = full;
  if (w < 2 || h < 2 || mipLevels < 2 || mipLevels > full || pImage->levelCount < mipLevels)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "the probe needs a %ux%u image (>= 2x2) with %u levels bound", w,
                h, mipLevels);
  const uint8_t* levels[NVPRO_PYRAMID_MAX_LEVELS];
  uint64_t pitches[NVPRO_PYRAMID_MAX_LEVELS];
  for (uint32_t k = 0; k < mipLevels; ++k) {
    levels[k] = static_cast<const uint8_t*>(pImage->levels[k]);
    pitches[k] = pImage->rowPitchBytes[k] ? pImage->rowPitchBytes[k] : uint64_t(levelDim(w, k)) * 4;
    if (!levels[k] || reinterpret_cast<uintptr_t>(levels[k]) % 4 || pitches[k] % 4)
      return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "level %u: null or not 4-byte aligned", k);
  }
  const cudaError_t e = launchProbe(levels, pitches, w, h, mipLevels, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "probe launch failed: %s", cudaGetErrorString(e));
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidPremultiplyAlpha(NvproPyramidStream stream, const void* src, uint64_t srcPitch,
                                               void* dst, uint64_t dstPitch, uint32_t width, uint32_t height) {
  if (!src || !dst) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "null image");
  if (width == 0 || height == 0) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "zero width or height");
  if (!srcPitch) srcPitch = uint64_t(width) * 4;
  if (!dstPitch) dstPitch = uint64_t(width) * 4;
  if (srcPitch < uint64_t(width) * 4 || dstPitch < uint64_t(width) * 4)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "row pitch below 4 * width");
  if ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst) | srcPitch | dstPitch) % 4)
    return fail(NVPRO_PYRAMID_ERROR_UNSUPPORTED, "texels must be 4-byte aligned");
  // in place (same pointer and pitch) or disjoint byte ranges; a partial overlap would race
  if (src != dst || srcPitch != dstPitch) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(src), b = reinterpret_cast<uintptr_t>(dst);
    const uint64_t aBytes = srcPitch * (height - 1) + uint64_t(width) * 4;
    const uint64_t bBytes = dstPitch * (height - 1) + uint64_t(width) * 4;
    if (a < b + bBytes && b < a + aBytes)
      return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "source and destination overlap without being equal");
  }
  const cudaError_t e = launchPremultiply(static_cast<const uint8_t*>(src), srcPitch, static_cast<uint8_t*>(dst),
                                          dstPitch, width, height, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "premultiply launch failed: %s", cudaGetErrorString(e));
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidDebugSrgbEncode(NvproPyramidStream stream, const float* x, uint8_t* fast,
                                               uint8_t* exact, uint64_t n) {
  if (!x || !fast || !exact) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "NULL buffer");
  cudaError_t e = launchDebugEncode(x, fast, exact, n, 0, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "debug encode: %s", cudaGetErrorString(e));
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidDebugAlphaEncode(NvproPyramidStream stream, const float* x, uint8_t* fast,
                                                uint8_t* exact, uint64_t n) {
  if (!x || !fast || !exact) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "NULL buffer");
  cudaError_t e = launchDebugEncode(x, fast, exact, n, 1, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "debug encode: %s", cudaGetErrorString(e));
  return NVPRO_PYRAMID_SUCCESS;
}

}  // extern "C"

namespace {

// The default dispatch schedule (nvpro_pyramid_dispatch.hpp:109-304 with a
// fast pipeline): isFast, input level and level count of each dispatch.
struct SchedEntry {
  uint32_t isFast, level, count, groups;
};

uint32_t defaultSchedule(uint32_t w, uint32_t h, uint32_t mipLevels, SchedEntry* out) {
  uint32_t n = 0;
  NvproPyramidState st{0u, mipLevels - 1u, w, h};
  while (st.remainingLevels != 0) {
    uint32_t done = 0, groups = 0, fast = 0;
    if (st.currentX % 4 == 0 && st.currentY % 4 == 0) {  // nvproPyramidDefaultFastDispatcher<4, 6>
      uint32_t x = st.currentX, y = st.currentY;
      while (x % 2 == 0 && y % 2 == 0 && done < st.remainingLevels && done < 6) {
        x /= 2;
        y /= 2;
        ++done;
      }
      fast = 1;
      const uint32_t shift = done > 5 ? 12u : 10u, mask = done > 5 ? 4095u : 1023u;
      groups = (st.currentX * st.currentY + mask) >> shift;
    } else {  // nvproPyramidDefaultGeneralDispatcher
      done = st.remainingLevels >= 2 ? 2u : st.remainingLevels;
      const uint32_t dw = std::max(st.currentX >> done, 1u), dh = std::max(st.currentY >> done, 1u);
      groups = done == 1 ? (dw * dh + 127) / 128 : ((dw + 7) / 8) * ((dh + 7) / 8);
    }
    out[n++] = SchedEntry{fast, st.currentLevel, done, groups};
    st.currentLevel += done;
    st.remainingLevels -= done;
    st.currentX = std::max(st.currentX >> done, 1u);
    st.currentY = std::max(st.currentY >> done, 1u);
  }
  return n;
}

// The default schedule of one image (nvpro_pyramid_dispatch.hpp:109-304 with
// both pipelines: nvproPyramidDefaultFastDispatcher<4, 6>, else
// nvproPyramidDefaultGeneralDispatcher) as launch parameters, in a
// caller-provided array of NVPRO_PYRAMID_MAX_LEVELS entries.
NvproPyramidResult defaultParams(NvproPyramidPreset preset, const NvproPyramidImage* pImage, uint32_t mipLevels,
                                 DispatchParams* params, uint32_t* count) {
  *count = 0;
  if (!pImage) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "pImage is NULL");
  if (presetBytes(uint32_t(preset)) == 0)
    return fail(NVPRO_PYRAMID_ERROR_UNSUPPORTED, "unknown preset %d", int(preset));
  const uint32_t w = pImage->width, h = pImage->height;
  if (w == 0 || h == 0) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "zero width or height");
  const uint32_t full = nvproPyramidFullLevelCount(w, h);
  if (mipLevels == 0) mipLevels = full;
  if (mipLevels > full || mipLevels > NVPRO_PYRAMID_MAX_LEVELS || pImage->levelCount < mipLevels)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "%u levels requested; %ux%u image binds %u of at most %u",
                mipLevels, w, h, pImage->levelCount, full);
  Record rec;
  std::memset(&rec, 0, sizeof rec);
  rec.image = *pImage;
  rec.info.preset = uint32_t(preset);
  rec.texelBytes = presetBytes(uint32_t(preset));
  rec.info.groupCountY = rec.info.groupCountZ = 1;
  SchedEntry sched[NVPRO_PYRAMID_MAX_LEVELS];
  const uint32_t n = defaultSchedule(w, h, mipLevels, sched);
  for (uint32_t i = 0; i < n; ++i) {
    rec.info.isFastPipeline = sched[i].isFast;
    rec.info.pushConstant = sched[i].level << NVPRO_PYRAMID_INPUT_LEVEL_SHIFT | sched[i].count;
    rec.info.groupCountX = sched[i].groups;
    NvproPyramidResult r = makeParams(rec, &params[i]);
    if (r != NVPRO_PYRAMID_SUCCESS) return r;
  }
  *count = n;
  return NVPRO_PYRAMID_SUCCESS;
}

// Levels whose adjoint values the sweep materialises in the workspace (all
// input levels of dispatches except 0, and the middle level of 2-level
// general dispatches), with their byte offsets.
uint64_t adjointWorkspaceLayout(uint32_t w, uint32_t h, uint32_t mipLevels, uint64_t* offsets) {
  SchedEntry sched[NVPRO_PYRAMID_MAX_LEVELS];
  const uint32_t n = defaultSchedule(w, h, mipLevels, sched);
  bool need[NVPRO_PYRAMID_MAX_LEVELS] = {};
  for (uint32_t i = 0; i < n; ++i) {
    if (sched[i].level > 0) need[sched[i].level] = true;
    if (!sched[i].isFast && sched[i].count == 2) need[sched[i].level + 1] = true;
  }
  uint64_t off = 0;
  for (uint32_t k = 0; k < mipLevels; ++k) {
    offsets[k] = need[k] ? off : UINT64_MAX;
    if (need[k]) off += uint64_t(levelDim(w, k)) * levelDim(h, k) * 16;
  }
  return off;
}

}  // namespace

extern "C" {

uint64_t nvproPyramidAdjointWorkspaceBytes(uint32_t width, uint32_t height, uint32_t mipLevels) {
  const uint32_t full = nvproPyramidFullLevelCount(width, height);
  if (width == 0 || height == 0) return 0;
  if (mipLevels == 0) mipLevels = full;
  if (mipLevels > full) return 0;
  uint64_t offsets[NVPRO_PYRAMID_MAX_LEVELS];
  return adjointWorkspaceLayout(width, height, mipLevels, offsets);
}

NvproPyramidResult nvproPyramidAdjoint(NvproPyramidStream stream, NvproPyramidPreset preset,
                                       const NvproPyramidImage* upstream, void* baseGrad, uint64_t baseGradPitch,
                                       uint32_t mipLevels, void* workspace, uint64_t workspaceBytes) {
  return nvproPyramidAdjointStrided(stream, preset, upstream, nullptr, baseGrad, baseGradPitch, 0, 1, mipLevels,
                                    workspace, workspaceBytes);
}

NvproPyramidResult nvproPyramidAdjointStrided(NvproPyramidStream stream, NvproPyramidPreset preset,
                                              const NvproPyramidImage* upstream, const uint64_t* upstreamImageStrides,
                                              void* baseGrad, uint64_t baseGradPitch, uint64_t baseGradImageStride,
                                              uint32_t count, uint32_t mipLevels, void* workspace,
                                              uint64_t workspaceBytes) {
  if (count == 0) return NVPRO_PYRAMID_SUCCESS;
  if (count > 65535) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "%u images: at most 65535", count);
  if (count > 1 && !upstreamImageStrides)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "upstreamImageStrides is NULL");
  if (preset != NVPRO_PYRAMID_PRESET_RGBA32F && preset != NVPRO_PYRAMID_PRESET_RGBA16F)
    return fail(NVPRO_PYRAMID_ERROR_UNSUPPORTED, "the adjoint exists for the linear float presets only");
  if (!upstream || !baseGrad) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "NULL upstream or baseGrad");
  const uint32_t w = upstream->width, h = upstream->height;
  const uint32_t full = nvproPyramidFullLevelCount(w, h);
  if (w == 0 || h == 0) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "zero width or height");
  if (mipLevels == 0) mipLevels = full;
  if (mipLevels > full || upstream->levelCount < mipLevels)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "%u levels requested; upstream binds %u of at most %u",
                mipLevels, upstream->levelCount, full);
  const uint32_t bpp = presetBytes(uint32_t(preset));
  const uint32_t gType = preset == NVPRO_PYRAMID_PRESET_RGBA32F ? 0u : 1u;
  if (baseGradPitch == 0) baseGradPitch = uint64_t(w) * bpp;
  if (baseGradPitch < uint64_t(w) * bpp || baseGradPitch % bpp || reinterpret_cast<uintptr_t>(baseGrad) % bpp)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "baseGrad pitch/alignment invalid");
  for (uint32_t k = 0; k < mipLevels; ++k) {
    const uint64_t pitch = upstream->rowPitchBytes[k] ? upstream->rowPitchBytes[k] : uint64_t(levelDim(w, k)) * bpp;
    if (upstream->levels[k] &&
        (reinterpret_cast<uintptr_t>(upstream->levels[k]) % bpp || pitch % bpp || pitch < uint64_t(levelDim(w, k)) * bpp))
      return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "upstream level %u pitch/alignment invalid", k);
  }
  uint64_t stride[NVPRO_PYRAMID_MAX_LEVELS] = {};
  for (uint32_t k = 0; k < mipLevels && count > 1; ++k) {
    stride[k] = upstreamImageStrides[k];
    if (stride[k] % bpp) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "image stride of level %u", k);
  }
  if (count > 1 && baseGradImageStride % bpp)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "baseGrad image stride is not a texel multiple");
  uint64_t wsOff[NVPRO_PYRAMID_MAX_LEVELS];
  const uint64_t wsImage = adjointWorkspaceLayout(w, h, mipLevels, wsOff);  // one image's share
  const uint64_t wsNeed = wsImage * count;
  if (wsNeed > workspaceBytes || (wsNeed && (!workspace || reinterpret_cast<uintptr_t>(workspace) % 16)))
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "workspace of %llu bytes (16-byte aligned) needed, got %llu",
                (unsigned long long)wsNeed, (unsigned long long)workspaceBytes);
  if (mipLevels == 1) {  // no levels above the base: the gradient is the upstream one
    const uint64_t rowBytes = uint64_t(w) * bpp;
    const uint64_t srcPitch = upstream->rowPitchBytes[0] ? upstream->rowPitchBytes[0] : rowBytes;
    cudaError_t e = cudaSuccess;
    for (uint32_t i = 0; i < count && e == cudaSuccess; ++i) {
      uint8_t* dst = static_cast<uint8_t*>(baseGrad) + i * baseGradImageStride;
      e = upstream->levels[0]
              ? cudaMemcpy2DAsync(dst, baseGradPitch, static_cast<const uint8_t*>(upstream->levels[0]) + i * stride[0],
                                  srcPitch, rowBytes, h, cudaMemcpyDeviceToDevice,
                                  reinterpret_cast<cudaStream_t>(stream))
              : cudaMemset2DAsync(dst, baseGradPitch, 0, rowBytes, h, reinterpret_cast<cudaStream_t>(stream));
    }
    return e == cudaSuccess ? NVPRO_PYRAMID_SUCCESS : fail(NVPRO_PYRAMID_ERROR_CUDA, "%s", cudaGetErrorString(e));
  }
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  uint8_t* ws = static_cast<uint8_t*>(workspace);
  // Where h_k lives: level 0 -> baseGrad; materialised levels -> workspace;
  // the top level -> the upstream gradient itself.
  auto hPtr = [&](uint32_t k) { return k == 0 ? static_cast<uint8_t*>(baseGrad) : ws + wsOff[k]; };
  auto hPitch = [&](uint32_t k) { return k == 0 ? baseGradPitch : uint64_t(levelDim(w, k)) * 16; };
  auto hType = [&](uint32_t k) { return k == 0 ? gType : 0u; };
  auto hImage = [&](uint32_t k) { return k == 0 ? baseGradImageStride : wsImage; };
  auto gPtr = [&](uint32_t k) { return static_cast<const uint8_t*>(upstream->levels[k]); };
  auto gPitch = [&](uint32_t k) {
    return upstream->rowPitchBytes[k] ? upstream->rowPitchBytes[k] : uint64_t(levelDim(w, k)) * bpp;
  };
  SchedEntry sched[NVPRO_PYRAMID_MAX_LEVELS];
  const uint32_t n = defaultSchedule(w, h, mipLevels, sched);
  const uint32_t top = mipLevels - 1;
  for (int i = int(n) - 1; i >= 0; --i) {
    const SchedEntry& d = sched[i];
    const uint32_t L = d.level, hi = d.level + d.count;
    // h of level `hi`: the upstream gradient if it is the top level
    const uint8_t* srcTop = hi == top ? gPtr(top) : hPtr(hi);
    const uint64_t srcPitch = hi == top ? gPitch(top) : hPitch(hi);
    const uint32_t srcType = hi == top ? gType : 0u;
    const uint64_t srcImage = hi == top ? stride[top] : wsImage;
    cudaError_t e;
    if (d.isFast) {
      AdjointChainParams p{};
      p.n = d.count;
      p.w = levelDim(w, L);
      p.h = levelDim(h, L);
      p.gType = gType;
      for (uint32_t k = 0; k < d.count; ++k) {
        p.g[k] = gPtr(L + k);
        p.gPitch[k] = gPitch(L + k);
      }
      p.top = srcTop;
      p.topPitch = srcPitch;
      p.topType = srcType;
      p.out = hPtr(L);
      p.outPitch = hPitch(L);
      p.outType = hType(L);
      p.batch = count;
      for (uint32_t k = 0; k < d.count; ++k) p.gImage[k] = stride[L + k];
      p.topImage = srcImage;
      p.outImage = hImage(L);
      e = launchAdjointChain(p, s);
    } else {
      e = cudaSuccess;
      const uint8_t* hc = srcTop;
      uint64_t hcPitch = srcPitch;
      uint32_t hcType = srcType;
      uint64_t hcImage = srcImage;
      for (int k = int(hi) - 1; k >= int(L) && e == cudaSuccess; --k) {
        AdjointLevelParams p{};
        p.fw = levelDim(w, k);
        p.fh = levelDim(h, k);
        p.cw = levelDim(w, k + 1);
        p.ch = levelDim(h, k + 1);
        p.g = gPtr(k);
        p.gPitch = gPitch(k);
        p.gType = gType;
        p.hc = hc;
        p.hcPitch = hcPitch;
        p.hcType = hcType;
        p.out = hPtr(k);
        p.outPitch = hPitch(k);
        p.outType = hType(k);
        p.batch = count;
        p.gImage = stride[k];
        p.hcImage = hcImage;
        p.outImage = hImage(k);
        e = launchAdjointLevel(p, s);
        hc = hPtr(k);
        hcPitch = hPitch(k);
        hcType = hType(k);
        hcImage = hImage(k);
      }
    }
    if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "adjoint launch failed: %s", cudaGetErrorString(e));
  }
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidGenerateNoAlloc(NvproPyramidStream stream, NvproPyramidPreset preset,
                                               const NvproPyramidImage* pImage, uint32_t mipLevels) {
  // The default schedule is built in fixed-size stack arrays: no command
  // object, no device or host allocation on the way to the launches.
  DispatchParams params[NVPRO_PYRAMID_MAX_LEVELS];
  uint32_t count = 0;
  NvproPyramidResult r = defaultParams(preset, pImage, mipLevels, params, &count);
  if (r != NVPRO_PYRAMID_SUCCESS) return r;
  if (count == 0) return NVPRO_PYRAMID_SUCCESS;

  // Plan every launch and its words of the fixed array before enqueueing
  // anything, so a rejected chain leaves the stream untouched.
  LaunchPlan plan[NVPRO_PYRAMID_MAX_LEVELS];
  const uint32_t launchCount = planLaunches(params, count, true, false, plan);
  uint32_t firstWord[NVPRO_PYRAMID_MAX_LEVELS];
  uint32_t words = kStaticErrorWord + 1;
  for (uint32_t k = 0; k < launchCount; ++k) {
    firstWord[k] = words;
    words += plan[k].words();
  }
  if (words > kStaticScratchWords)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "chain needs %u of the %u fixed scratch words", words,
                kStaticScratchWords);

  uint32_t* scratch = nullptr;
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = staticScratch(&scratch);
  // Calls share the array and it keeps the last call's contents: the counters
  // start from zero; the error word stays until the status query reads it.
  if (e == cudaSuccess && words > kStaticErrorWord + 1)
    e = cudaMemsetAsync(scratch + kStaticErrorWord + 1, 0, (words - kStaticErrorWord - 1) * sizeof(uint32_t), s);
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "static scratch: %s", cudaGetErrorString(e));
  uint32_t launches = 0;
  for (uint32_t k = 0; k < launchCount && e == cudaSuccess; ++k)
    e = runLaunch(plan[k], params, s, Scratch{scratch + firstWord[k], plan[k].words(), scratch + kStaticErrorWord},
                  &launches);
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidNoAllocDeviceStatus(NvproPyramidStream stream) {
  uint32_t* scratch = nullptr;
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = staticScratch(&scratch);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  uint32_t flag = 0;  // read into the stack: nothing is allocated
  if (e == cudaSuccess) e = cudaMemcpy(&flag, scratch + kStaticErrorWord, sizeof flag, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && flag) {
    e = cudaMemsetAsync(scratch + kStaticErrorWord, 0, sizeof flag, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "no-alloc device status: %s", cudaGetErrorString(e));
  if (flag) return fail(NVPRO_PYRAMID_ERROR_TIMEOUT, "a device-side wait gave up; outputs are incomplete");
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidDebugNoAllocForceWaitTimeout(NvproPyramidStream stream, uint32_t waitKind) {
  if (waitKind > 1) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "waitKind %u", waitKind);
  uint32_t* scratch = nullptr;
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = staticScratch(&scratch);
  // the counters of a general launch at the first per-launch word, the error word shared
  const Scratch sc{scratch + kStaticErrorWord + 1, kGeneralScratchWords, scratch + kStaticErrorWord};
  if (e == cudaSuccess && waitKind == 1) e = cudaMemsetAsync(sc.counters, 0, kGeneralScratchWords * 4, s);
  if (e == cudaSuccess) e = waitKind == 0 ? launchDebugMbarTimeout(sc.error(), s) : launchDebugGridBarrierTimeout(sc, s);
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "launch failed: %s", cudaGetErrorString(e));
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidGenerate(NvproPyramidCmd cmd, NvproPyramidStream stream,
                                        NvproPyramidPipelines pipelines, const NvproPyramidImage* pImage,
                                        uint32_t mipLevels) {
  NvproPyramidResult r = nvproPyramidBeginCmd(cmd, stream);
  if (r != NVPRO_PYRAMID_SUCCESS) return r;
  nvproPyramidCmdBindImage(cmd, pImage);
  if (pImage) nvproCmdPyramidDispatch(cmd, pipelines, pImage->width, pImage->height, mipLevels);
  return nvproPyramidEndCmd(cmd);
}

NvproPyramidResult nvproPyramidGenerateStrided(NvproPyramidCmd cmd, NvproPyramidStream stream,
                                               NvproPyramidPipelines pipelines, const NvproPyramidImage* pImage,
                                               const uint64_t* imageStrides, uint32_t count, uint32_t mipLevels) {
  if (!validCmd(cmd)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid command object");
  if (count == 0) return NVPRO_PYRAMID_SUCCESS;
  if (count > 65535) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "%u images: at most 65535", count);
  if (count > 1 && !imageStrides) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "imageStrides is NULL");
  if (count > 1 && pImage) {
    const uint32_t bpp = validPipeline(pipelines.generalPipeline) ? pipelines.generalPipeline->texelBytes : 0;
    for (uint32_t k = 0; k < pImage->levelCount && k < NVPRO_PYRAMID_MAX_LEVELS; ++k)
      if (bpp && imageStrides[k] % bpp)
        return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "image stride of level %u is not a texel multiple", k);
  }
  cmd->batch = count;
  for (uint32_t k = 0; k < NVPRO_PYRAMID_MAX_LEVELS; ++k)
    cmd->imageStrides[k] = count > 1 && pImage && k < pImage->levelCount ? imageStrides[k] : 0;
  const NvproPyramidResult r = nvproPyramidGenerate(cmd, stream, pipelines, pImage, mipLevels);
  cmd->batch = 1;
  std::memset(cmd->imageStrides, 0, sizeof cmd->imageStrides);
  return r;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches (no reference counterpart): many images, one persistent launch.

namespace {

constexpr uint32_t kBatchMagic = 0x4E50424Du;  // 'NPBM'

// The autotuner's candidates per axis (coordinate descent from the default
// tuple, one axis after the other).  The reference's precedent is the offline
// sweep of workgroup and tile sizes of extras/general_pipelines/
// py2_generate_all.py:9-10 and the fixed choice it led to
// (nvpro_pyramid_dispatch.hpp:254-258).  Levels per dispatch are not an axis:
// they are the default dispatcher's (nvproPyramidDefaultFastDispatcher<4, 6>),
// and other values would change the bytes.
constexpr uint32_t kBandCandidates[] = {4, 8, 16, 32};
constexpr uint32_t kRowsCandidates[] = {16, 32, 64};
constexpr uint32_t kWarpsCandidates[] = {8, 12};

// Autotuner cache: the tuple by size class (GPU name, mip levels and the
// histogram of log2(max side) over the batch, counts rounded to powers of
// two), in memory and in a text file that later processes read
// (sizeClassKey, tuneCacheFile).
std::mutex g_tuneMu;
std::map<std::string, BatchTuning> g_tuneCache;

std::string sizeClassKey(const NvproPyramidImage* images, uint32_t count, uint32_t mipLevels) {
  uint32_t hist[32] = {};
  for (uint32_t i = 0; i < count; ++i) {
    uint32_t m = std::max(images[i].width, images[i].height), b = 0;
    while (m >>= 1) ++b;
    ++hist[b];
  }
  int dev = 0;
  cudaDeviceProp prop{};
  std::string gpu = "gpu";
  if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess) gpu = prop.name;
  for (char& c : gpu)
    if (c == ' ' || c == '\t' || c == '\n') c = '_';
  std::string key = gpu + ":" + std::to_string(mipLevels) + ":";
  for (uint32_t b = 0; b < 32; ++b) {
    uint32_t c = hist[b], r = 0;
    while (c) {
      c >>= 1;
      ++r;
    }
    key += char('a' + r);
  }
  return key;
}

// The cache file: NVPRO_PYRAMID_CACHE_DIR, else $XDG_CACHE_HOME/nvpro_pyramid,
// else $HOME/.cache/nvpro_pyramid; "" if none can be named.
std::string tuneCacheFile() {
  std::string dir;
  if (const char* d = std::getenv("NVPRO_PYRAMID_CACHE_DIR")) {
    dir = d;
  } else if (const char* x = std::getenv("XDG_CACHE_HOME")) {
    dir = std::string(x) + "/nvpro_pyramid";
  } else if (const char* h = std::getenv("HOME")) {
    dir = std::string(h) + "/.cache/nvpro_pyramid";
  }
  return dir.empty() ? dir : dir + "/batch_tuning.txt";
}

// One line per tuned size class: "<key> <band> <rows> <warps>"; the last
// line of a key wins.  A missing or unreadable file is an empty cache.
bool readTuneCache(const std::string& key, BatchTuning* t) {
  const std::string path = tuneCacheFile();
  if (path.empty()) return false;
  FILE* f = std::fopen(path.c_str(), "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (std::fgets(line, sizeof line, f)) {
    char k[400];
    unsigned band = 0, rows = 0, warps = 0;
    if (std::sscanf(line, "%399s %u %u %u", k, &band, &rows, &warps) == 4 && key == k && band >= 1 &&
        band <= 4096 && (rows == 16 || rows == 32 || rows == 64) && (warps == 8 || warps == 12)) {
      *t = BatchTuning{band, rows, warps};
      found = true;
    }
  }
  std::fclose(f);
  return found;
}

// Append a tuned size class (best effort: no directory or no permission
// leaves the in-memory cache only).  One write of one short line.
void writeTuneCache(const std::string& key, const BatchTuning& t) {
  const std::string path = tuneCacheFile();
  if (path.empty()) return;
  const std::string dir = path.substr(0, path.rfind('/'));
  mkdir(dir.c_str(), 0755);  // one level; its parent is expected to exist
  FILE* f = std::fopen(path.c_str(), "a");
  if (!f) return;
  std::fprintf(f, "%s %u %u %u\n", key.c_str(), t.stripBand, t.fastRows, t.warps);
  std::fclose(f);
}

}  // namespace

struct NvproPyramidBatch_T {
  uint32_t magic = kBatchMagic;
  NvproPyramidPreset preset = NVPRO_PYRAMID_PRESET_SRGBA8;
  uint32_t flags = 0;
  nvpyr::BatchPlan plan;
  nvpyr::BatchDevice dev;
  void* devMem = nullptr;
  uint64_t devBytes = 0;
  uint32_t imageCount = 0;
  BatchTuning tuning;
  BatchTuning fixed{0, 0, 0};  // nvproPyramidBatchSetTuning: non-zero fields override default and autotuner
  uint32_t autotuned = 0, fromCache = 0, fromDisk = 0;
  cudaStream_t captureStream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool built = false;

  void dropGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
  ~NvproPyramidBatch_T() {
    dropGraph();
    if (captureStream) cudaStreamDestroy(captureStream);
    if (devMem) cudaFree(devMem);
    magic = 0;
  }
  // the tuple with the fixed fields applied
  BatchTuning withFixed(BatchTuning t) const {
    if (fixed.stripBand) t.stripBand = fixed.stripBand;
    if (fixed.fastRows) t.fastRows = fixed.fastRows;
    if (fixed.warps) t.warps = fixed.warps;
    return t;
  }
  // plan with `tuning` and copy it to the device block (grown if needed)
  cudaError_t planAndUpload(const std::vector<std::vector<DispatchParams>>& imgs, const BatchTuning& t,
                            cudaStream_t s) {
    cudaError_t e = plan.build(imgs, t);
    if (e != cudaSuccess) return e;
    const uint64_t need = plan.deviceBytes();
    if (need > devBytes) {
      if (devMem) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        cudaFree(devMem);
        devMem = nullptr;
        devBytes = 0;
      }
      e = cudaMalloc(&devMem, need);
      if (e != cudaSuccess) return e;
      devBytes = need;
      e = cudaMemset(devMem, 0, need);  // the error flag starts clear
      if (e != cudaSuccess) return e;
    }
    e = plan.upload(devMem, s, &dev);
    dev.warps = t.warps;
    return e;
  }
  // median of five timed launches (after two untimed) of the current plan
  cudaError_t time(cudaStream_t s, cudaEvent_t* ev, float* ms) {
    constexpr int kWarm = 2, kTimed = 5;
    float t[kTimed] = {};
    uint32_t launches = 0;
    cudaError_t e = cudaSuccess;
    for (int it = 0; it < kWarm + kTimed && e == cudaSuccess; ++it) {
      const bool timed = it >= kWarm;
      if (timed) e = cudaEventRecord(ev[0], s);
      if (e == cudaSuccess) e = nvpyr::launchBatch(dev, s, &launches);
      if (e == cudaSuccess && timed) e = cudaEventRecord(ev[1], s);
      if (e == cudaSuccess && timed) e = cudaEventSynchronize(ev[1]);
      if (e == cudaSuccess && timed) e = cudaEventElapsedTime(&t[it - kWarm], ev[0], ev[1]);
    }
    std::sort(t, t + kTimed);
    *ms = t[kTimed / 2];
    return e;
  }
  // coordinate descent over the candidates of the axes that are not fixed
  cudaError_t autotune(const std::vector<std::vector<DispatchParams>>& imgs, cudaStream_t s, BatchTuning* best) {
    cudaEvent_t ev[2];
    cudaError_t e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    BatchTuning cur = withFixed(BatchTuning{});
    float bestMs = 0;
    auto tryTuple = [&](const BatchTuning& t) {
      float ms = 0;
      if (e == cudaSuccess) e = planAndUpload(imgs, t, s);
      if (e == cudaSuccess) e = time(s, ev, &ms);
      if (e == cudaSuccess && (bestMs == 0 || ms < bestMs)) {
        bestMs = ms;
        cur = t;
      }
    };
    tryTuple(cur);
    if (!fixed.stripBand)
      for (uint32_t b : kBandCandidates)
        if (b != cur.stripBand) tryTuple(BatchTuning{b, cur.fastRows, cur.warps});
    if (!fixed.fastRows)
      for (uint32_t r : kRowsCandidates)
        if (r != cur.fastRows) tryTuple(BatchTuning{cur.stripBand, r, cur.warps});
    if (!fixed.warps)
      for (uint32_t w : kWarpsCandidates)
        if (w != cur.warps) tryTuple(BatchTuning{cur.stripBand, cur.fastRows, w});
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    *best = cur;
    return e;
  }
};

namespace {
bool validBatch(NvproPyramidBatch b) { return b && b->magic == kBatchMagic; }
}  // namespace

extern "C" {

NvproPyramidResult nvproPyramidCreateBatch(NvproPyramidPreset preset, uint32_t flags, NvproPyramidBatch* pBatch) {
  if (!pBatch) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "pBatch is NULL");
  *pBatch = nullptr;
  if (preset != NVPRO_PYRAMID_PRESET_SRGBA8)
    return fail(NVPRO_PYRAMID_ERROR_UNSUPPORTED, "batches exist for the sRGBA8 preset only");
  if (flags & ~(NVPRO_PYRAMID_BATCH_AUTOTUNE | NVPRO_PYRAMID_BATCH_GRAPH | NVPRO_PYRAMID_BATCH_RETUNE))
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "unknown batch flags 0x%x", flags);
  auto* b = new (std::nothrow) NvproPyramidBatch_T;
  if (!b) return fail(NVPRO_PYRAMID_ERROR_OUT_OF_MEMORY, "batch object");
  b->preset = preset;
  b->flags = flags;
  *pBatch = b;
  return NVPRO_PYRAMID_SUCCESS;
}

void nvproPyramidDestroyBatch(NvproPyramidBatch batch) {
  if (validBatch(batch)) delete batch;
}

NvproPyramidResult nvproPyramidBatchBuild(NvproPyramidBatch b, NvproPyramidStream stream,
                                          const NvproPyramidImage* images, uint32_t imageCount,
                                          uint32_t mipLevels) {
  if (!validBatch(b)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid batch object");
  if (!images && imageCount) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "images is NULL");
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  b->built = false;
  b->dropGraph();
  std::vector<std::vector<DispatchParams>> imgs(imageCount);
  for (uint32_t i = 0; i < imageCount; ++i) {
    DispatchParams params[NVPRO_PYRAMID_MAX_LEVELS];
    uint32_t count = 0;
    NvproPyramidResult r = defaultParams(b->preset, &images[i], mipLevels, params, &count);
    if (r != NVPRO_PYRAMID_SUCCESS) return r;
    imgs[i].assign(params, params + count);
  }
  b->imageCount = imageCount;
  b->autotuned = b->fromCache = b->fromDisk = 0;
  BatchTuning tuning = b->withFixed(BatchTuning{});
  cudaError_t e = cudaSuccess;
  const bool allFixed = b->fixed.stripBand && b->fixed.fastRows && b->fixed.warps;
  if ((b->flags & NVPRO_PYRAMID_BATCH_AUTOTUNE) && !allFixed) {
    const std::string key = sizeClassKey(images, imageCount, mipLevels);
    bool cached = false;
    if (!(b->flags & NVPRO_PYRAMID_BATCH_RETUNE)) {
      std::lock_guard<std::mutex> lock(g_tuneMu);
      auto it = g_tuneCache.find(key);
      if (it != g_tuneCache.end()) {
        tuning = b->withFixed(it->second);
        cached = true;
      } else if (readTuneCache(key, &tuning)) {
        g_tuneCache[key] = tuning;
        tuning = b->withFixed(tuning);
        cached = true;
        b->fromDisk = 1;
      }
    }
    if (!cached) {
      // Time the candidates on `stream` -- the real work, writing the images' levels.
      e = b->autotune(imgs, s, &tuning);
      if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "batch autotune: %s", cudaGetErrorString(e));
      std::lock_guard<std::mutex> lock(g_tuneMu);
      g_tuneCache[key] = tuning;
      writeTuneCache(key, tuning);
    }
    b->autotuned = 1;
    b->fromCache = cached ? 1 : 0;
  }
  b->tuning = tuning;
  e = b->planAndUpload(imgs, tuning, s);
  if (e == cudaErrorInvalidValue)
    return fail(NVPRO_PYRAMID_ERROR_UNSUPPORTED, "a dispatch of the batch is not supported by the batch kernel");
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "batch tables: %s", cudaGetErrorString(e));
  if (b->flags & NVPRO_PYRAMID_BATCH_GRAPH) {
    // Capture the launch (counter reset + kernel) once; launches replay it.
    e = nvpyr::batchDeviceReady();
    if (e == cudaSuccess && !b->captureStream) e = cudaStreamCreateWithFlags(&b->captureStream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(b->captureStream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      uint32_t launches = 0;
      const cudaError_t le = nvpyr::launchBatch(b->dev, b->captureStream, &launches);
      e = cudaStreamEndCapture(b->captureStream, &b->graph);
      if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) {
      b->dropGraph();
      return fail(NVPRO_PYRAMID_ERROR_CUDA, "batch graph: %s", cudaGetErrorString(e));
    }
  }
  b->built = true;
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidBatchSetStripBand(NvproPyramidBatch b, uint32_t band) {
  if (!validBatch(b)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid batch object");
  return nvproPyramidBatchSetTuning(b, band, b->fixed.fastRows, b->fixed.warps * 32);
}

NvproPyramidResult nvproPyramidBatchSetTuning(NvproPyramidBatch b, uint32_t stripBand, uint32_t fastRegionRows,
                                              uint32_t threadsPerCta) {
  if (!validBatch(b)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid batch object");
  if (stripBand > 4096) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "strip band %u > 4096", stripBand);
  if (fastRegionRows != 0 && fastRegionRows != 16 && fastRegionRows != 32 && fastRegionRows != 64)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "fast region rows %u: 16, 32 or 64", fastRegionRows);
  if (threadsPerCta != 0 && threadsPerCta != 256 && threadsPerCta != 384)
    return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "threads per CTA %u: 256 or 384", threadsPerCta);
  b->fixed = BatchTuning{stripBand, fastRegionRows, threadsPerCta / 32};
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidBatchLaunch(NvproPyramidBatch b, NvproPyramidStream stream) {
  if (!validBatch(b)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid batch object");
  if (!b->built) return fail(NVPRO_PYRAMID_ERROR_INVALID_STATE, "batch is not built");
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (b->exec) {
    e = cudaGraphLaunch(b->exec, s);
  } else {
    uint32_t launches = 0;
    e = nvpyr::launchBatch(b->dev, s, &launches);
  }
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "batch launch: %s", cudaGetErrorString(e));
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidBatchGetInfo(NvproPyramidBatch b, NvproPyramidBatchInfo* info) {
  if (!validBatch(b) || !info) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid batch or info");
  std::memset(info, 0, sizeof *info);
  info->imageCount = b->imageCount;
  info->phaseCount = b->plan.phaseCount();
  info->jobCount = b->plan.jobCount();
  info->stripBand = b->tuning.stripBand;
  info->fastRegionRows = b->tuning.fastRows;
  info->threadsPerCta = b->tuning.warps * 32;
  info->fromDisk = b->fromDisk;
  info->unitCount = b->plan.unitCount();
  info->autotuned = b->autotuned;
  info->fromCache = b->fromCache;
  info->graph = b->exec ? 1u : 0u;
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidBatchDeviceStatus(NvproPyramidBatch b) {
  if (!validBatch(b)) return fail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "invalid batch object");
  if (!b->built || !b->dev.counters) return NVPRO_PYRAMID_SUCCESS;
  cudaError_t e = cudaDeviceSynchronize();
  uint32_t flag = 0;
  uint8_t* at = reinterpret_cast<uint8_t*>(b->dev.counters) + b->plan.errorFlagOffset();
  if (e == cudaSuccess) e = cudaMemcpy(&flag, at, sizeof flag, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && flag) e = cudaMemset(at, 0, sizeof flag);
  if (e != cudaSuccess) return fail(NVPRO_PYRAMID_ERROR_CUDA, "batch status: %s", cudaGetErrorString(e));
  if (flag) return fail(NVPRO_PYRAMID_ERROR_TIMEOUT, "a bounded device wait of the batch kernel gave up");
  return NVPRO_PYRAMID_SUCCESS;
}

}  // extern "C"
