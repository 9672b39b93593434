/*
 * nvpro_pyramid_cuda.h -- C ABI of the GB300 image-pyramid (mipmap) engine.
 *
 * This is the drop-in replacement for the host side of nvpro_pyramid
 * (nvpro_pyramid/nvpro_pyramid_dispatch.hpp in nvpro-samples/vk_compute_mipmaps).
 * The reference records Vulkan compute dispatches onto a VkCommandBuffer; this
 * library records the same dispatch sequence into an NvproPyramidCmd and, at
 * nvproPyramidEndCmd, launches CUDA kernels for sm_103a onto a CUDA stream.
 *
 * Mapping of reference concepts:
 *   VkCommandBuffer            -> NvproPyramidCmd (recorder bound to a cudaStream_t)
 *   VkPipeline (fast/general)  -> NvproPyramidPipeline (preset + fast/general kernels)
 *   descriptor sets            -> NvproPyramidImage (per-level device pointers)
 *   push constant (4 bytes)    -> nvproPyramidCmdPushConstants, same encoding
 *                                 (inputLevel << 5 | levelCount)
 *   vkCmdDispatch              -> nvproPyramidCmdDispatch (same workgroup counts)
 *   vkCmdPipelineBarrier       -> nvproPyramidCmdPipelineBarrier (stream order)
 *   assert() in the dispatcher -> NvproPyramidResult error codes
 *
 * All functions are plain C: no C++ or torch types cross this boundary.
 * Device memory is owned by the caller; the library allocates device memory
 * only in nvproPyramidCreateCmd (a few bytes of counters), never while
 * recording or launching.
 */
#ifndef NVPRO_PYRAMID_CUDA_H_
#define NVPRO_PYRAMID_CUDA_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define NVPRO_PYRAMID_API __declspec(dllexport)
#else
#define NVPRO_PYRAMID_API __attribute__((visibility("default")))
#endif

/* A CUDA stream (cudaStream_t / CUstream); NULL is the legacy default stream. */
typedef struct CUstream_st* NvproPyramidStream;

/* Replaces the reference's assert()s (nvpro_pyramid_dispatch.hpp:169,172). */
typedef enum NvproPyramidResult {
  NVPRO_PYRAMID_SUCCESS                = 0,
  NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT = 1, /* null pointer, bad size, level out of range */
  NVPRO_PYRAMID_ERROR_INVALID_STATE    = 2, /* e.g. dispatch with no bound pipeline or image */
  NVPRO_PYRAMID_ERROR_DISPATCHER       = 3, /* dispatcher returned 0 or more than remainingLevels */
  NVPRO_PYRAMID_ERROR_UNSUPPORTED      = 4, /* preset / layout not supported by a kernel */
  NVPRO_PYRAMID_ERROR_CUDA             = 5, /* a CUDA runtime call failed */
  NVPRO_PYRAMID_ERROR_OUT_OF_MEMORY    = 6,
  NVPRO_PYRAMID_ERROR_TIMEOUT          = 7, /* a bounded device-side wait gave up */
  NVPRO_PYRAMID_ERROR_IO               = 8  /* a file could not be read or written */
} NvproPyramidResult;

/* Static description of a result code. */
NVPRO_PYRAMID_API const char* nvproPyramidResultString(NvproPyramidResult result);
/* Human-readable detail of the last error raised on the calling thread ("" if none). */
NVPRO_PYRAMID_API const char* nvproPyramidLastError(void);

/* ------------------------------------------------------------------------ */
/* Pipelines.  The reference compiles one fast and one general VkPipeline    */
/* per preset (srgba8_mipmap_{fast,general}_pipeline.comp); here a pipeline  */
/* names a preset and which of the two kernel families it runs.              */
/* ------------------------------------------------------------------------ */

typedef enum NvproPyramidPreset {
  /* nvpro_pyramid/srgba8_mipmap_preamble.glsl:10-128: RGBA8 texels, RGB
   * sRGB-encoded, alpha linear; reductions in linear FP32; 4 bytes/texel. */
  NVPRO_PYRAMID_PRESET_SRGBA8  = 1,
  /* Linear RGBA FP32 texels (16 bytes/texel).  No reference preset; the
   * template admits any NVPRO_PYRAMID_TYPE (nvpro_pyramid.glsl:44-46). */
  NVPRO_PYRAMID_PRESET_RGBA32F = 2,
  /* Linear RGBA FP16 storage (8 bytes/texel), FP32 arithmetic. */
  NVPRO_PYRAMID_PRESET_RGBA16F = 3
} NvproPyramidPreset;

typedef struct NvproPyramidPipeline_T* NvproPyramidPipeline;

/* Create the fast (isFastPipeline != 0; nvpro_pyramid.glsl:209-534) or the
 * general (nvpro_pyramid.glsl:536-885) pipeline of a preset.  Replaces the
 * vkCreateComputePipelines calls of minimal_app/minimal_mipmaps.cpp:178-190. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCreatePipeline(
    NvproPyramidPreset preset, uint32_t isFastPipeline, NvproPyramidPipeline* pPipeline);

/* Pipeline configuration bits: the macros the reference's demo prepends to
 * the shader source per pipeline (demo_app/mipmap_pipelines.cpp:107-122),
 * with the values of demo_app/pipeline_alternative.hpp:38-43.
 *
 * SRGB_SHARED / F16_SHARED (srgba8_mipmap_preamble.glsl:60-108; sRGBA8
 * preset only, at most one of the two): the values a dispatch hands from one
 * level to the next through shared memory are kept in a compact format.  Those
 * are level L+3 of a fast dispatch of 4 or 5 levels, level L+4 of a 6-level
 * fast dispatch (sharedTile_, nvpro_pyramid.glsl:253,395,487-512) and level
 * L+1 of a 2-level general dispatch (sharedLevel_, :555,664,717).  The levels
 * after the hand-off are reduced from the compact values; the hand-off level
 * itself is stored from its FP32 values, as in the reference.
 *   SRGB_SHARED: the texel's sRGBA8 code (the preset's own store encoding)
 *   decoded again with the preset's load tables.  The reference's srgbPack /
 *   srgbUnpack compute the same code with pow() and packUnorm4x8, whose
 *   precision and rounding of halves GLSL leaves to the implementation; the
 *   exact codec is the pinned reading.
 *   F16_SHARED: each channel rounded to binary16 (round to nearest even).
 *
 * NO_BILINEAR (srgba8_mipmap_preamble.glsl:40-58): LOAD_REDUCE4 as four
 * texel loads instead of one bilinear sample.  Every pipeline of this library
 * computes it that way (hardware bilinear filtering precision is
 * implementation-defined), so the bit is accepted and changes nothing. */
#define NVPRO_PYRAMID_CONFIG_SRGB_SHARED 0x1u
#define NVPRO_PYRAMID_CONFIG_F16_SHARED  0x2u
#define NVPRO_PYRAMID_CONFIG_NO_BILINEAR 0x4u

/* nvproPyramidCreatePipeline with configuration bits (0 = the default
 * pipeline).  UNSUPPORTED for a shared format on a preset other than sRGBA8;
 * INVALID_ARGUMENT for both shared formats or an unknown bit. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCreatePipelineEx(
    NvproPyramidPreset preset, uint32_t isFastPipeline, uint32_t configBits, NvproPyramidPipeline* pPipeline);
NVPRO_PYRAMID_API void nvproPyramidDestroyPipeline(NvproPyramidPipeline pipeline);

/* Bytes per texel of a preset (0 for an unknown preset). */
NVPRO_PYRAMID_API uint32_t nvproPyramidPresetTexelBytes(NvproPyramidPreset preset);

/* ------------------------------------------------------------------------ */
/* Custom pipelines: a caller's own texel format and reduction (the          */
/* reference's customisation macros, nvpro_pyramid.glsl:27-120).  The C++    */
/* header nvpro_pyramid_cuda.hpp makes them from a device-functor set        */
/* (nvpro_pyramid::createPipelines<F>); at this level a pipeline is a        */
/* launcher that runs one recorded dispatch.                                 */
/* ------------------------------------------------------------------------ */

/* The preset value a custom pipeline reports in its dispatch records. */
#define NVPRO_PYRAMID_PRESET_CUSTOM 0x100u

/* One level of a dispatch: texel (0, 0) of image 0, row pitch, size, and the
 * bytes between the images of a strided call (0 for one image). */
typedef struct NvproPyramidLevelDesc {
  void*    texels;
  uint64_t rowPitchBytes;
  uint32_t width;
  uint32_t height;
  uint64_t imageStrideBytes;
} NvproPyramidLevelDesc;

/* One recorded dispatch, as the reference's shader sees it through its push
 * constant (inputLevel << 5 | levelCount) and its workgroup count. */
typedef struct NvproPyramidDispatchDesc {
  uint32_t isFastPipeline;
  uint32_t inputLevel;
  uint32_t levelCount;             /* levels filled: 1..6 (fast), 1..2 (general) */
  uint32_t imageCount;             /* images of the call (grid z of a strided call) */
  uint64_t groupCount;             /* workgroups dispatched (0 if any count was 0) */
  NvproPyramidLevelDesc levels[7]; /* levels inputLevel .. inputLevel + levelCount */
} NvproPyramidDispatchDesc;

/* Enqueue the kernels of one dispatch on `stream`; return NVPRO_PYRAMID_SUCCESS
 * or an error code (which nvproPyramidEndCmd returns). */
typedef NvproPyramidResult (*nvpro_pyramid_launcher_t)(void* userData, NvproPyramidStream stream,
                                                       const NvproPyramidDispatchDesc* dispatch);

/* A fast or general pipeline whose dispatches run through `launcher` (no
 * reference counterpart as a function: the reference compiles the caller's
 * shader into a VkPipeline).  Levels bound with it hold texelBytes bytes per
 * texel; their addresses and row pitches must be multiples of the largest
 * power of two dividing texelBytes (at most 16). */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCreateCustomPipeline(
    uint32_t isFastPipeline, uint32_t texelBytes, nvpro_pyramid_launcher_t launcher, void* userData,
    NvproPyramidPipeline* pPipeline);

/* NvproPyramidPipelines (nvpro_pyramid_dispatch.hpp:29-35).  `layout` is an
 * opaque caller pointer handed unchanged to the dispatcher callbacks (the
 * VkPipelineLayout slot); pushConstantOffset must be 0 (the 4-byte push
 * constant has no other home here). */
typedef struct NvproPyramidPipelines {
  NvproPyramidPipeline generalPipeline; /* mandatory */
  NvproPyramidPipeline fastPipeline;    /* optional (NULL) */
  const void*          layout;
  uint32_t             pushConstantOffset;
} NvproPyramidPipelines;

/* ------------------------------------------------------------------------ */
/* Images (the descriptor sets of srgba8_mipmap_preamble.glsl:10-13).        */
/* ------------------------------------------------------------------------ */

#define NVPRO_PYRAMID_MAX_LEVELS 32

/* Level k has size max(width >> k, 1) x max(height >> k, 1)
 * (nvpro_pyramid_dispatch.hpp:175-178; include/mipmap_storage.hpp:67-69).
 * levels[k] is the device address of texel (0,0) of level k; rows are
 * rowPitchBytes[k] apart (0 = tightly packed). */
typedef struct NvproPyramidImage {
  uint32_t width;
  uint32_t height;
  uint32_t levelCount; /* number of valid entries of levels[] */
  uint32_t reserved;
  void*    levels[NVPRO_PYRAMID_MAX_LEVELS];
  uint64_t rowPitchBytes[NVPRO_PYRAMID_MAX_LEVELS];
} NvproPyramidImage;

/* Number of levels of a full chain: floor(log2(max(w, h))) + 1
 * (nvpro_pyramid_dispatch.hpp:122-132).  0 if w == h == 0. */
NVPRO_PYRAMID_API uint32_t nvproPyramidFullLevelCount(uint32_t width, uint32_t height);

/* Byte offset of each level in the packed layout of MipmapStorage
 * (include/mipmap_storage.hpp:53-76): levels contiguous, each [y][x].
 * Writes levelCount + 1 offsets (the last one is the total size). */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidPackedLayout(
    uint32_t width, uint32_t height, uint32_t levelCount, uint32_t bytesPerTexel,
    uint64_t* pOffsets);

/* Fill an NvproPyramidImage for a packed allocation starting at `base`. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidImageInitPacked(
    NvproPyramidImage* pImage, void* base, uint32_t width, uint32_t height,
    uint32_t levelCount, uint32_t bytesPerTexel);

/* ------------------------------------------------------------------------ */
/* Command recording (VkCommandBuffer analogue).                             */
/* ------------------------------------------------------------------------ */

typedef struct NvproPyramidCmd_T* NvproPyramidCmd;

/* Record, but launch nothing at nvproPyramidEndCmd (no CUDA call at all). */
#define NVPRO_PYRAMID_CMD_RECORD_ONLY 0x1u
/* Launch one kernel per recorded dispatch (no in-kernel tail fusion). */
#define NVPRO_PYRAMID_CMD_NO_FUSION 0x2u
/* Use only the portable (plain load/store) kernels, never the TMA kernels. */
#define NVPRO_PYRAMID_CMD_PORTABLE_KERNELS 0x4u

/* A command object is externally synchronised, like a VkCommandBuffer: one
 * thread records it, and its launches must not overlap another submission of
 * the same object on the GPU (they share its device counters). */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCreateCmd(uint32_t flags, NvproPyramidCmd* pCmd);
NVPRO_PYRAMID_API void nvproPyramidDestroyCmd(NvproPyramidCmd cmd);

/* vkBeginCommandBuffer: clears previous records and binds the stream. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidBeginCmd(NvproPyramidCmd cmd, NvproPyramidStream stream);
/* vkEndCommandBuffer + vkQueueSubmit: lowers the recorded dispatches to
 * kernel launches on the stream.  Returns the first error raised while
 * recording, if any (then nothing is launched). */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidEndCmd(NvproPyramidCmd cmd);

/* vkCmdBindDescriptorSets: the image every later dispatch reads and writes. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCmdBindImage(NvproPyramidCmd cmd, const NvproPyramidImage* pImage);
/* vkCmdBindPipeline (nvpro_pyramid_dispatch.hpp:213,262). */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCmdBindPipeline(NvproPyramidCmd cmd, NvproPyramidPipeline pipeline);
/* vkCmdPushConstants (nvpro_pyramid_dispatch.hpp:231,269): 4 bytes at offset 0. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCmdPushConstants(
    NvproPyramidCmd cmd, const void* layout, uint32_t offset, uint32_t size, const void* pValues);
/* vkCmdDispatch (nvpro_pyramid_dispatch.hpp:238,282,289).  Workgroup counts
 * have the reference's meaning (fast: 256-thread groups over 1024 or 4096
 * input samples; general: 128 outputs or one 8x8 tile of the second level);
 * a smaller count leaves the reference's uncovered texels unwritten. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCmdDispatch(
    NvproPyramidCmd cmd, uint32_t groupCountX, uint32_t groupCountY, uint32_t groupCountZ);
/* vkCmdBlitImage of level srcLevel to level srcLevel + 1 of the bound image
 * with VK_FILTER_LINEAR (the fallback of the demo's "generalblit" mode,
 * demo_app/mipmap_pipelines.cpp:350-452), in the texel format of the bound
 * pipeline's preset.  Destination texel (x, y) samples the source at
 * ((x + 0.5) * srcW / dstW, (y + 0.5) * srcH / dstH) with a bilinear filter
 * on decoded (linear) values, clamped to the edge, and is stored with the
 * preset's encoding.  The blit's filter precision is the Vulkan
 * implementation's; here it is FP32, each operation rounded: scale =
 * srcW / dstW, u = (x + 0.5) * scale - 0.5, i = floor(u), a = u - i;
 * rows lerped first (t0 * (1 - a) + t1 * a), then the column. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCmdBlitLevel(NvproPyramidCmd cmd, uint32_t srcLevel);

/* vkCmdPipelineBarrier (nvpro_pyramid_dispatch.hpp:183-186). */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCmdPipelineBarrier(NvproPyramidCmd cmd);

/* One recorded dispatch, for inspection and tests. */
typedef struct NvproPyramidDispatchRecord {
  uint32_t isFastPipeline;
  uint32_t preset;
  uint32_t pushConstant; /* inputLevel << 5 | levelCount */
  uint32_t groupCountX;
  uint32_t groupCountY;
  uint32_t groupCountZ;
  uint32_t pipelineBound;  /* a bind preceded this dispatch */
  uint32_t barrierBefore;  /* a barrier preceded this dispatch */
  uint32_t configBits;     /* NVPRO_PYRAMID_CONFIG_* of the bound pipeline */
  uint32_t isBlit;         /* a blit (nvproPyramidCmdBlitLevel), not a dispatch */
} NvproPyramidDispatchRecord;

NVPRO_PYRAMID_API uint32_t nvproPyramidCmdRecordCount(NvproPyramidCmd cmd);
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCmdGetRecords(
    NvproPyramidCmd cmd, NvproPyramidDispatchRecord* pRecords, uint32_t count);
/* Kernel launches issued by the last nvproPyramidEndCmd. */
NVPRO_PYRAMID_API uint32_t nvproPyramidCmdLaunchCount(NvproPyramidCmd cmd);

/* Wait for the command's stream, then report NVPRO_PYRAMID_ERROR_TIMEOUT if a
 * bounded device-side wait of one of its kernels gave up since the last query
 * (the outputs of that submission are then incomplete).  Clears the report.
 * No reference counterpart: Vulkan reports device loss instead. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCmdDeviceStatus(NvproPyramidCmd cmd);

/* Speed-of-light probe (the reference's "baseline" general-pipeline
 * alternative, extras/general_pipelines/baseline/
 * general_pipeline_alternative.glsl:1-26): one launch with the memory traffic
 * of a whole sRGBA8 chain (level 0 read once, levels 1 .. mipLevels-1 written
 * once) and no filtering, as a roofline calibration.  The levels it writes
 * are NOT a pyramid.  Image >= 2x2; mipLevels 0 = all. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidSpeedOfLightProbe(
    NvproPyramidStream stream, const NvproPyramidImage* pImage, uint32_t mipLevels);

/* Premultiplied-alpha staging (the -do-premultiply-alpha path of
 * minimal_app/minimal_mipmaps.cpp:316-367, done by the reference on the host
 * in include/scoped_image.hpp:233-255): every sRGBA8 texel of a width x height
 * image in DEVICE memory becomes (enc(dec(r) * a), enc(dec(g) * a),
 * enc(dec(b) * a), A) with a = A * (1.0f / 255.0f) in FP32, dec the exact sRGB
 * decode and enc the exact sRGB encode of the pyramid kernels.  src == dst
 * (in place) is allowed; pitches 0 mean 4 * width.  Asynchronous on stream. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidPremultiplyAlpha(
    NvproPyramidStream stream, const void* src, uint64_t srcPitch, void* dst, uint64_t dstPitch,
    uint32_t width, uint32_t height);

/* Test support for failure detection (no reference counterpart): launch, on
 * the command's stream, one small kernel whose bounded device-side wait runs
 * out -- waitKind 0: the fast kernel's mbarrier wait on a phase nothing
 * completes; 1: the general chain's grid barrier that nothing releases.  It
 * gives up after its limit (about a second) and sets the command's error
 * flag, so the next nvproPyramidCmdDeviceStatus reports
 * NVPRO_PYRAMID_ERROR_TIMEOUT and resets the counters; nothing faults.
 * waitKind 2 launches nothing: in the command's next TMA fast-kernel launch,
 * CTA 0 takes the path of a wait that gave up at once (its regions stay
 * unwritten, the fused tail is skipped, the error flag is set) while the
 * kernel's own counter still returns to zero, so later launches are correct
 * before any status query. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidDebugForceWaitTimeout(NvproPyramidCmd cmd, uint32_t waitKind);

/* Test support (no reference counterpart): encode n floats of x (device
 * memory) with the kernels' fast sRGB encoder into `fast` (inputs clamped to
 * its domain [0, 1] first), and with the exact threshold count into `exact`. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidDebugSrgbEncode(
    NvproPyramidStream stream, const float* x, uint8_t* fast, uint8_t* exact, uint64_t n);

/* Test support (no reference counterpart): the alpha byte of the kernels'
 * texel encoder for each float of x (clamped to [0, 1] first) into `fast`, and
 * clamp(uint(a * 255 + 0.5), 0, 255) with separately rounded operations
 * (srgba8_mipmap_preamble.glsl:125) into `exact`. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidDebugAlphaEncode(
    NvproPyramidStream stream, const float* x, uint8_t* fast, uint8_t* exact, uint64_t n);

/* ------------------------------------------------------------------------ */
/* The dispatcher (nvpro_pyramid_dispatch.hpp:54-304).                       */
/* ------------------------------------------------------------------------ */

#define NVPRO_PYRAMID_INPUT_LEVEL_SHIFT 5u /* nvproPyramidInputLevelShift, :77 */

/* NvproPyramidState (nvpro_pyramid_dispatch.hpp:63-75). */
typedef struct NvproPyramidState {
  uint32_t currentLevel;
  uint32_t remainingLevels;
  uint32_t currentX;
  uint32_t currentY;
} NvproPyramidState;

/* nvpro_pyramid_dispatcher_t (nvpro_pyramid_dispatch.hpp:99-104): record one
 * bind (if pipelineIfNeeded != NULL), push constant and dispatch; return the
 * number of levels filled.  A fast dispatcher may return 0 to decline; a
 * general dispatcher must not. */
typedef uint32_t (*nvpro_pyramid_dispatcher_t)(
    NvproPyramidCmd cmdBuf, const void* layout, uint32_t pushConstantOffset,
    NvproPyramidPipeline pipelineIfNeeded, const NvproPyramidState* state);

/* nvproCmdPyramidDispatch with the default dispatchers
 * (nvpro_pyramid_dispatch.hpp:54-59, :294-304).  mipLevels == 0 means the
 * full chain.  Requires a bound image with at least mipLevels levels. */
NVPRO_PYRAMID_API NvproPyramidResult nvproCmdPyramidDispatch(
    NvproPyramidCmd cmdBuf, NvproPyramidPipelines pipelines, uint32_t baseWidth,
    uint32_t baseHeight, uint32_t mipLevels);

/* The base overload with caller dispatchers (nvpro_pyramid_dispatch.hpp:109-188). */
NVPRO_PYRAMID_API NvproPyramidResult nvproCmdPyramidDispatchEx(
    NvproPyramidCmd cmdBuf, NvproPyramidPipelines pipelines, uint32_t baseWidth,
    uint32_t baseHeight, uint32_t mipLevels, nvpro_pyramid_dispatcher_t generalDispatcher,
    nvpro_pyramid_dispatcher_t fastDispatcher);

/* nvproPyramidDefaultFastDispatcher<4, 6> (nvpro_pyramid_dispatch.hpp:195-242). */
NVPRO_PYRAMID_API uint32_t nvproPyramidDefaultFastDispatcher(
    NvproPyramidCmd cmdBuf, const void* layout, uint32_t pushConstantOffset,
    NvproPyramidPipeline pipelineIfNeeded, const NvproPyramidState* state);

/* The body of nvproPyramidDefaultFastDispatcher<DivisibilityRequirement,
 * MaxLevels> for any even DivisibilityRequirement and MaxLevels in 1..6, for
 * C callers that cannot instantiate the template (e.g. the <2, 5> and <2, 6>
 * variants registered in demo_app/nvpro_pyramid_dispatch_alternative.cpp:41-42). */
NVPRO_PYRAMID_API uint32_t nvproPyramidFastDispatch(
    NvproPyramidCmd cmdBuf, const void* layout, uint32_t pushConstantOffset,
    NvproPyramidPipeline pipelineIfNeeded, const NvproPyramidState* state,
    uint32_t divisibilityRequirement, uint32_t maxLevels);

/* nvproPyramidDefaultGeneralDispatcher (nvpro_pyramid_dispatch.hpp:247-292). */
NVPRO_PYRAMID_API uint32_t nvproPyramidDefaultGeneralDispatcher(
    NvproPyramidCmd cmdBuf, const void* layout, uint32_t pushConstantOffset,
    NvproPyramidPipeline pipelineIfNeeded, const NvproPyramidState* state);

/* A general dispatcher that blits one level instead of dispatching the
 * general pipeline (it binds pipelineIfNeeded when given, for the preset):
 * nvproCmdPyramidDispatchEx with it and nvproPyramidDefaultFastDispatcher is
 * the demo's "generalblit" mode -- the fast pipeline where the sizes allow
 * it, a linear blit of one level otherwise (demo_app/mipmap_pipelines.cpp:
 * 350-452, pipeline_alternative.cpp:16).  Returns 1. */
NVPRO_PYRAMID_API uint32_t nvproPyramidBlitGeneralDispatcher(
    NvproPyramidCmd cmdBuf, const void* layout, uint32_t pushConstantOffset,
    NvproPyramidPipeline pipelineIfNeeded, const NvproPyramidState* state);

/* Begin + bind image + nvproCmdPyramidDispatch + End in one call: the whole
 * sequence of minimal_app/minimal_mipmaps.cpp:199-210 (bind descriptor sets,
 * dispatch, submit) for callers that record nothing else.  The image's
 * width/height are the base size. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidGenerate(
    NvproPyramidCmd cmd, NvproPyramidStream stream, NvproPyramidPipelines pipelines,
    const NvproPyramidImage* pImage, uint32_t mipLevels);

/* nvproPyramidGenerate for `count` images of the same size and layout (no
 * reference counterpart): image i's level k is image->levels[k] + i *
 * imageStrides[k] (bytes).  Every dispatch is one launch over all images (the
 * portable kernels, image = grid z): for many float images, e.g. a
 * [B, H, W, 4] tensor per level. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidGenerateStrided(
    NvproPyramidCmd cmd, NvproPyramidStream stream, NvproPyramidPipelines pipelines,
    const NvproPyramidImage* image, const uint64_t* imageStrides, uint32_t count, uint32_t mipLevels);

/* ------------------------------------------------------------------------ */
/* Adjoint of the linear float pyramids.  No reference counterpart (the      */
/* reference template admits float types, nvpro_pyramid.glsl:44-46, but has  */
/* no gradient).                                                             */
/* ------------------------------------------------------------------------ */

/* Bytes of FP32 workspace nvproPyramidAdjoint needs for a w x h chain of
 * mipLevels levels (0 = full chain): the intermediate levels of the sweep. */
NVPRO_PYRAMID_API uint64_t nvproPyramidAdjointWorkspaceBytes(uint32_t width, uint32_t height,
                                                             uint32_t mipLevels);

/* Gradient of sum_k <upstream_k, level_k> with respect to the base level, for
 * the RGBA32F or RGBA16F preset (FP32 arithmetic).  `upstream` holds the
 * upstream gradient of every level in the preset's storage type
 * (upstream->levels[k] may be NULL: zero gradient); the result is written to
 * baseGrad (preset storage type, row pitch baseGradPitch or tightly packed if
 * 0).  The sweep follows the forward's default dispatch schedule coarse to
 * fine; each texel of baseGrad is written once.  workspace: device memory of
 * nvproPyramidAdjointWorkspaceBytes bytes, 16-byte aligned. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidAdjoint(
    NvproPyramidStream stream, NvproPyramidPreset preset, const NvproPyramidImage* upstream,
    void* baseGrad, uint64_t baseGradPitch, uint32_t mipLevels, void* workspace,
    uint64_t workspaceBytes);

/* nvproPyramidAdjoint for `count` images of the same size (no reference
 * counterpart): image i's upstream level k is upstream->levels[k] + i *
 * upstreamImageStrides[k] (bytes; may be NULL when count == 1), its base
 * gradient baseGrad + i * baseGradImageStride; the workspace holds count times
 * nvproPyramidAdjointWorkspaceBytes.  One launch per dispatch for all images. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidAdjointStrided(
    NvproPyramidStream stream, NvproPyramidPreset preset, const NvproPyramidImage* upstream,
    const uint64_t* upstreamImageStrides, void* baseGrad, uint64_t baseGradPitch, uint64_t baseGradImageStride,
    uint32_t count, uint32_t mipLevels, void* workspace, uint64_t workspaceBytes);

/* The whole default chain (both pipelines of `preset`, mipLevels == 0 for the
 * full chain) on `stream`, without allocating anything.  No counterpart in the
 * reference.
 *
 * For callers that cannot allocate device memory: code running where a host
 * application owns every device allocation (plugins, fixed memory budgets),
 * and hot loops that must not call cudaMalloc/cudaFree (cudaFree synchronises
 * the device).  nvproPyramidCreateCmd allocates a few bytes of device counters;
 * this entry point instead uses a fixed 1 KiB __device__ array of the library
 * (256 words: one error word, then two per TMA launch and five per run of
 * general dispatches of the chain; a chain has at most 31 dispatches, so every
 * chain fits, and the words a chain needs are checked before anything is
 * enqueued).  Every GPU that loads the library holds the array until the
 * process exits.
 *
 * The first call on a device (and again after the device's context was made
 * anew, e.g. after cudaDeviceReset) looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls share the array and it keeps the last
 * call's contents: each call clears its launch counters on `stream` first,
 * while the error word keeps a timed-out wait of any call until
 * nvproPyramidNoAllocDeviceStatus reads it.  Calls whose work overlaps on the
 * GPU (e.g. on two streams without ordering) race on the array: order them. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidGenerateNoAlloc(
    NvproPyramidStream stream, NvproPyramidPreset preset, const NvproPyramidImage* pImage,
    uint32_t mipLevels);

/* The device status of nvproPyramidGenerateNoAlloc, allocating nothing (the
 * no-allocation counterpart of nvproPyramidCmdDeviceStatus): wait for
 * `stream`, then report NVPRO_PYRAMID_ERROR_TIMEOUT if a bounded device-side
 * wait of a kernel launched by nvproPyramidGenerateNoAlloc (on any stream of
 * the current device) gave up since the last query -- the outputs of that call
 * are then incomplete -- and clear the report. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidNoAllocDeviceStatus(NvproPyramidStream stream);

/* Test support (no reference counterpart): nvproPyramidDebugForceWaitTimeout
 * on the fixed array of nvproPyramidGenerateNoAlloc, on `stream`: the next
 * nvproPyramidNoAllocDeviceStatus reports NVPRO_PYRAMID_ERROR_TIMEOUT. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidDebugNoAllocForceWaitTimeout(NvproPyramidStream stream,
                                                                             uint32_t waitKind);

/* ------------------------------------------------------------------------ */
/* Batches (no reference counterpart: the reference records one chain per   */
/* command buffer, nvpro_pyramid_dispatch.hpp:109-188, and its benchmark     */
/* submits images one at a time, demo_app/mipmaps_app.cpp:666-767).         */
/*                                                                          */
/* A batch generates the full default chain of many sRGBA8 images of any    */
/* sizes in one persistent kernel launch: phase k runs the k-th dispatch of */
/* every image's schedule, warps take work units from a per-phase queue,    */
/* and a grid barrier separates phases.  The bytes equal those of           */
/* nvproPyramidGenerate on each image.                                       */
/* ------------------------------------------------------------------------ */

typedef struct NvproPyramidBatch_T* NvproPyramidBatch;

/* Build flags. */
#define NVPRO_PYRAMID_BATCH_AUTOTUNE 1u /* pick the launch's shape (strip band, fast-region rows,
                                           threads per CTA) by timing candidates, cached per size
                                           class of the batch in memory and on disk */
#define NVPRO_PYRAMID_BATCH_GRAPH 2u    /* launches replay a CUDA graph captured at build */
#define NVPRO_PYRAMID_BATCH_RETUNE 4u   /* with AUTOTUNE: time the candidates even if a cache has
                                           the size class (and store the new choice) */

typedef struct NvproPyramidBatchInfo {
  uint32_t imageCount;
  uint32_t phaseCount;     /* dispatches of the longest schedule */
  uint32_t jobCount;       /* dispatches over all images */
  uint32_t stripBand;      /* rows of level L+2 per general-pipeline work unit */
  uint64_t unitCount;      /* work units over all phases */
  uint32_t autotuned;      /* the shape was chosen by the autotuner */
  uint32_t fromCache;      /* ... from a cache (an earlier build of the same size class) */
  uint32_t graph;          /* launches replay a CUDA graph */
  uint32_t fastRegionRows; /* rows of level L per fast-pipeline work unit (64 texels wide) */
  uint32_t threadsPerCta;  /* 256 or 384 */
  uint32_t fromDisk;       /* the cached shape came from the cache file of an earlier process */
} NvproPyramidBatchInfo;

NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidCreateBatch(NvproPyramidPreset preset, uint32_t flags,
                                                             NvproPyramidBatch* pBatch);
NVPRO_PYRAMID_API void nvproPyramidDestroyBatch(NvproPyramidBatch batch);

/* Plan the batch for `images` (each with its levels bound as for
 * nvproPyramidGenerate; mipLevels as there, 0 = each image's full chain) and
 * copy the plan to device memory that the batch owns.  With
 * NVPRO_PYRAMID_BATCH_AUTOTUNE and a size class not seen before, this runs
 * the batch a few times on `stream` (writing the images' levels) and waits
 * for it.  The image memory must stay valid while the batch is launched. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidBatchBuild(NvproPyramidBatch batch, NvproPyramidStream stream,
                                                            const NvproPyramidImage* images,
                                                            uint32_t imageCount, uint32_t mipLevels);

/* Fix the work-unit size of general-pipeline dispatches (rows of level L+2
 * per strip; 0 = the default, or the autotuner's choice with
 * NVPRO_PYRAMID_BATCH_AUTOTUNE) for the following nvproPyramidBatchBuild. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidBatchSetStripBand(NvproPyramidBatch batch, uint32_t band);

/* Fix any of the launch's shape parameters for the following
 * nvproPyramidBatchBuild (0 = default, or the autotuner's choice): the strip
 * band (1..4096), the rows of level L per fast-pipeline region (16, 32 or 64;
 * at least 2^n for an n-level dispatch) and the threads per CTA (256 or 384).
 * The shape never changes the bytes written.  The autotuner's cache file is
 * NVPRO_PYRAMID_CACHE_DIR/batch_tuning.txt (else $XDG_CACHE_HOME/nvpro_pyramid
 * or $HOME/.cache/nvpro_pyramid), one line per size class and GPU name. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidBatchSetTuning(NvproPyramidBatch batch, uint32_t stripBand,
                                                                uint32_t fastRegionRows, uint32_t threadsPerCta);

/* Generate levels 1.. of every image of the batch on `stream` (no
 * allocation, no host synchronisation).  Launches of one batch must not
 * overlap on the GPU: they share the batch's work counters. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidBatchLaunch(NvproPyramidBatch batch, NvproPyramidStream stream);

NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidBatchGetInfo(NvproPyramidBatch batch,
                                                              NvproPyramidBatchInfo* info);

/* Wait for the device, then report NVPRO_PYRAMID_ERROR_TIMEOUT if a bounded
 * grid-barrier wait of a launch of this batch gave up since the last query. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidBatchDeviceStatus(NvproPyramidBatch batch);

/* ------------------------------------------------------------------------ */
/* Debugging I/O of sRGBA8 levels in HOST memory (no CUDA call).             */
/* ------------------------------------------------------------------------ */

/* One level (RGBA8 rows rowPitchBytes apart; 0 = 4 * width) as an
 * uncompressed 32-bit TGA file, top-left origin. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidWriteTga(const char* path, const void* rgba8, uint32_t width,
                                                          uint32_t height, uint64_t rowPitchBytes);

/* writeMipmapsTga (include/mipmap_storage.hpp:436-479): levelCount levels
 * (0 = all) of a packed chain (nvproPyramidPackedLayout, 4 bytes per texel)
 * to TGA files: level 0 to baseFilename, level k to baseFilename with ".k"
 * inserted before its extension ("out.tga" -> "out.3.tga"). */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidWriteLevelsTga(const char* baseFilename, const void* packed,
                                                                uint32_t width, uint32_t height,
                                                                uint32_t levelCount);

/* Read a 24- or 32-bit true-colour TGA (uncompressed or RLE, either vertical
 * origin) into top-left RGBA8 rows (alpha 255 for 24-bit files).  With
 * rgba8 == NULL only *pWidth / *pHeight are set; else capacityBytes must be
 * at least 4 * width * height. */
NVPRO_PYRAMID_API NvproPyramidResult nvproPyramidReadTga(const char* path, void* rgba8, uint64_t capacityBytes,
                                                         uint32_t* pWidth, uint32_t* pHeight);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* NVPRO_PYRAMID_CUDA_H_ */
