// kernels_stage.cu -- passes beside the pyramid: the premultiplied-alpha
// staging of sRGBA8 images (the reference's -do-premultiply-alpha staging,
// include/scoped_image.hpp:203-255, done there on the host per texel) and a
// speed-of-light probe of a chain's memory traffic.
//
// Premultiply, per texel: a = A * (1/255) (the reference's FP32 expression),
// each colour channel c -> encode(decode(c) * a), alpha byte unchanged.
// decode is the library's exact sRGB table and encode the exact threshold
// count (the codec of every pyramid kernel) where the reference uses FP32
// pow(); for all 65,536 (code, alpha) pairs the bytes are the reference's.
// The result depends on (c, A) only, so a 64 KiB table of all pairs is built
// once per device (premulTableKernel, into a file-scope __device__ array)
// and the pass is a stream over the image (4 bytes read and written per
// texel) with three byte lookups per texel from a shared-memory copy of the
// table: each thread moves 4 texels per 16-byte access, four accesses in
// flight.
#include <algorithm>
#include <mutex>

#include "srgb_codec.cuh"

namespace nvpyr {
namespace {

constexpr uint32_t kThreads = 512;
constexpr uint32_t kUnroll = 4;            // 16-byte accesses in flight per thread
constexpr uint32_t kSmemBytes = 1u << 16;  // the (alpha, code) -> premultiplied code table
constexpr float kInv255 = 1.0f / 255.0f;   // (1.F / 255.F) of scoped_image.hpp

// Premultiplied colour code of (code c, alpha A) at byte A << 8 | (c ^ s(A)),
// s(A) = (A & 31) << 2.  The swizzle makes the shared-memory bank of a lookup
// ((c >> 2) ^ A) mod 32 depend on both bytes: without it the bank is c >> 2
// alone, and texels of one dark or premultiplied colour but different alphas
// queue on one bank (an in-place pass over an already premultiplied image ran
// 3.4x slower).
static __device__ __align__(16) uint8_t g_premulTable[1u << 16];

__host__ __device__ __forceinline__ uint32_t premulSwizzle(uint32_t alpha) { return (alpha & 31u) << 2; }

__global__ void __launch_bounds__(256) premulTableKernel() {
  __shared__ SrgbTablesSmem tabs;
  loadSrgbTables(&tabs);
  __syncthreads();
  const uint32_t alpha = blockIdx.x, c = threadIdx.x;  // 256 blocks of 256 codes
  const float a = __fmul_rn(__uint2float_rn(alpha), kInv255);
  g_premulTable[alpha << 8 | (c ^ premulSwizzle(alpha))] =
      uint8_t(srgbEncodeSearch(__fmul_rn(tabs.decode[c], a), tabs.thr));
}

struct PremulParams {
  const uint8_t* src;
  uint8_t* dst;
  uint64_t srcPitch, dstPitch;
  uint32_t width, height;
  uint32_t quadsPerRow;  // ceil(width / 4)
  uint32_t vec;          // 1: rows and pointers 16-byte aligned, whole quads use 16-byte accesses
};

// A colour channel of texel t through the table at shared address `tab`: one
// PRMT forms A << 8 | c (the selector picks the channel), `swz` = s(A).
__device__ __forceinline__ uint32_t premulChannel(uint32_t t, uint32_t tab, uint32_t swz, uint32_t selector) {
  uint32_t v;
  asm("ld.shared.u8 %0, [%1];" : "=r"(v) : "r"(tab + (__byte_perm(t, 0, selector) ^ swz)));
  return v;
}

__device__ __forceinline__ uint32_t premultiplyTexel(uint32_t t, uint32_t tab) {
  const uint32_t swz = premulSwizzle(t >> 24);
  const uint32_t r = premulChannel(t, tab, swz, 0x4430), g = premulChannel(t, tab, swz, 0x4431),
                 b = premulChannel(t, tab, swz, 0x4432);
  return __byte_perm(__byte_perm(r, g, 0x0040), __byte_perm(b, t, 0x0070), 0x5410);
}

__global__ void __launch_bounds__(kThreads, 3) premultiplyKernel(const PremulParams p) {
  extern __shared__ __align__(128) uint8_t smem[];
  for (uint32_t i = threadIdx.x; i < kSmemBytes / 16; i += kThreads)
    reinterpret_cast<uint4*>(smem)[i] = reinterpret_cast<const uint4*>(g_premulTable)[i];
  __syncthreads();
  const uint32_t tab = smemAddr(smem);
  const uint64_t quads = uint64_t(p.quadsPerRow) * p.height;
  const uint64_t stride = uint64_t(gridDim.x) * kThreads * kUnroll;
  for (uint64_t q0 = uint64_t(blockIdx.x) * kThreads * kUnroll + threadIdx.x; q0 < quads; q0 += stride) {
    uint4 t[kUnroll];
    uint32_t n[kUnroll];  // texels of each quad (0 past the end)
#pragma unroll
    for (uint32_t u = 0; u < kUnroll; ++u) {
      const uint64_t q = q0 + uint64_t(u) * kThreads;
      n[u] = 0;
      t[u] = make_uint4(0, 0, 0, 0);
      if (q >= quads) continue;
      const uint32_t y = uint32_t(q / p.quadsPerRow), x = uint32_t(q % p.quadsPerRow) * 4;
      n[u] = min(4u, p.width - x);
      const uint8_t* s = p.src + y * p.srcPitch + uint64_t(x) * 4;
      if (p.vec && n[u] == 4) {
        t[u] = __ldcs(reinterpret_cast<const uint4*>(s));
      } else {
        const uint32_t* s32 = reinterpret_cast<const uint32_t*>(s);
        t[u].x = s32[0];
        if (n[u] > 1) t[u].y = s32[1];
        if (n[u] > 2) t[u].z = s32[2];
        if (n[u] > 3) t[u].w = s32[3];
      }
    }
#pragma unroll
    for (uint32_t u = 0; u < kUnroll; ++u) {
      if (n[u] == 0) continue;
      const uint64_t q = q0 + uint64_t(u) * kThreads;
      const uint32_t y = uint32_t(q / p.quadsPerRow), x = uint32_t(q % p.quadsPerRow) * 4;
      const uint4 r = make_uint4(premultiplyTexel(t[u].x, tab), premultiplyTexel(t[u].y, tab),
                                 premultiplyTexel(t[u].z, tab), premultiplyTexel(t[u].w, tab));
      uint8_t* d = p.dst + y * p.dstPitch + uint64_t(x) * 4;
      if (p.vec && n[u] == 4) {
        __stcs(reinterpret_cast<uint4*>(d), r);
      } else {
        uint32_t* d32 = reinterpret_cast<uint32_t*>(d);
        d32[0] = r.x;
        if (n[u] > 1) d32[1] = r.y;
        if (n[u] > 2) d32[2] = r.z;
        if (n[u] > 3) d32[3] = r.w;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Speed-of-light probe (the reference's "baseline" general pipeline,
// extras/general_pipelines/baseline/general_pipeline_alternative.glsl:1-26):
// the memory traffic of a whole chain -- level 0 read once, every other level
// written once -- with no filtering, as a roofline calibration.  Thread t owns
// four texels of level 1 (x1 = 4 qx .. +3, row y1): it reads their 2x2 blocks
// of level 0 (two 32-byte row pieces), stores the byte-wise average of each
// block to level 1, and the same value to texel (x1 + j, y1) of every coarser
// level that has it, so each level's texels are written exactly once.  The
// output is deliberately not a pyramid.

struct ProbeParams {
  const uint8_t* l0;
  uint64_t pitch0;
  uint32_t h0;
  uint32_t levels;  // levels 1 .. levels - 1 are written
  uint8_t* lv[32];
  uint64_t pitch[32];
  uint32_t w[32], h[32];
  uint32_t quadsPerRow;  // ceil(w1 / 4)
  uint32_t vec;          // level 0 and level 1 rows 16-byte aligned
};

__device__ __forceinline__ uint32_t avg4(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  return __vavgu4(__vavgu4(a, b), __vavgu4(c, d));
}

__global__ void __launch_bounds__(256) probeKernel(const __grid_constant__ ProbeParams p) {
  const uint64_t quads = uint64_t(p.quadsPerRow) * p.h[1];
  for (uint64_t q = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < quads;
       q += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t y1 = uint32_t(q / p.quadsPerRow), x1 = uint32_t(q % p.quadsPerRow) * 4;
    const uint32_t n = min(4u, p.w[1] - x1);
    const uint8_t* r0 = p.l0 + uint64_t(2 * y1) * p.pitch0 + uint64_t(2 * x1) * 4;
    const uint8_t* r1 = 2 * y1 + 1 < p.h0 ? r0 + p.pitch0 : r0;
    uint32_t v[4];
    if (p.vec && n == 4) {
      const uint4 a0 = __ldcs(reinterpret_cast<const uint4*>(r0)), a1 = __ldcs(reinterpret_cast<const uint4*>(r0) + 1);
      const uint4 b0 = __ldcs(reinterpret_cast<const uint4*>(r1)), b1 = __ldcs(reinterpret_cast<const uint4*>(r1) + 1);
      v[0] = avg4(a0.x, a0.y, b0.x, b0.y);
      v[1] = avg4(a0.z, a0.w, b0.z, b0.w);
      v[2] = avg4(a1.x, a1.y, b1.x, b1.y);
      v[3] = avg4(a1.z, a1.w, b1.z, b1.w);
      *reinterpret_cast<uint4*>(p.lv[1] + uint64_t(y1) * p.pitch[1] + uint64_t(x1) * 4) =
          make_uint4(v[0], v[1], v[2], v[3]);
    } else {
      const uint32_t* a = reinterpret_cast<const uint32_t*>(r0);
      const uint32_t* b = reinterpret_cast<const uint32_t*>(r1);
      for (uint32_t j = 0; j < n; ++j) {
        v[j] = avg4(a[2 * j], a[2 * j + 1], b[2 * j], b[2 * j + 1]);
        reinterpret_cast<uint32_t*>(p.lv[1] + uint64_t(y1) * p.pitch[1])[x1 + j] = v[j];
      }
    }
    for (uint32_t k = 2; k < p.levels && y1 < p.h[k] && x1 < p.w[k]; ++k) {
      uint32_t* row = reinterpret_cast<uint32_t*>(p.lv[k] + uint64_t(y1) * p.pitch[k]);
      for (uint32_t j = 0; j < n && x1 + j < p.w[k]; ++j) row[x1 + j] = v[j];
    }
  }
}

struct StageDevice {
  int sms = 0;
  int premulCtas = 1;  // resident premultiply CTAs per SM
  bool table = false;  // g_premulTable filled on this device
};

// Device state; with `needTable`, fills the premultiply table on first use
// (on `stream`, then waits for it once, so that any stream may use it after).
cudaError_t stageDevice(int* sms, bool needTable = false, cudaStream_t stream = nullptr, int* premulCtas = nullptr) {
  static StageDevice devs[64];
  static std::mutex mu;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (devs[dev].sms == 0) {
    e = cudaFuncSetAttribute(premultiplyKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemBytes));
    // all of the unified L1/shared storage as shared memory, so that the
    // resident CTAs are bounded by the table copies, not by the carveout
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(premultiplyKernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                               int(cudaSharedmemCarveoutMaxShared));
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&devs[dev].premulCtas, premultiplyKernel, kThreads,
                                                        kSmemBytes);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&devs[dev].sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  if (needTable && !devs[dev].table) {
    premulTableKernel<<<256, 256, 0, stream>>>();
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return e;
    devs[dev].table = true;
  }
  *sms = devs[dev].sms;
  if (premulCtas) *premulCtas = std::max(devs[dev].premulCtas, 1);
  return cudaSuccess;
}

}  // namespace

cudaError_t launchProbe(const uint8_t* const* levels, const uint64_t* pitches, uint32_t width, uint32_t height,
                        uint32_t levelCount, cudaStream_t stream) {
  if (levelCount < 2 || levelCount > 32) return cudaErrorInvalidValue;
  int sms = 0;
  cudaError_t e = stageDevice(&sms);
  if (e != cudaSuccess) return e;
  ProbeParams p{};
  p.l0 = levels[0];
  p.pitch0 = pitches[0];
  p.h0 = height;
  p.levels = levelCount;
  for (uint32_t k = 0; k < levelCount; ++k) {
    p.lv[k] = const_cast<uint8_t*>(levels[k]);
    p.pitch[k] = pitches[k];
    p.w[k] = std::max(width >> k, 1u);
    p.h[k] = std::max(height >> k, 1u);
  }
  if (width < 2 || height < 2) return cudaErrorInvalidValue;  // a 2x2 block per level-1 texel
  p.quadsPerRow = (p.w[1] + 3) / 4;
  p.vec = (reinterpret_cast<uintptr_t>(p.l0) | reinterpret_cast<uintptr_t>(p.lv[1]) | p.pitch0 | p.pitch[1]) % 16 == 0;
  const uint64_t quads = uint64_t(p.quadsPerRow) * p.h[1];
  const uint32_t grid = uint32_t(std::min<uint64_t>((quads + 255) / 256, uint64_t(sms) * 16));
  probeKernel<<<grid, 256, 0, stream>>>(p);
  return cudaGetLastError();
}

cudaError_t launchPremultiply(const uint8_t* src, uint64_t srcPitch, uint8_t* dst, uint64_t dstPitch, uint32_t width,
                              uint32_t height, cudaStream_t stream) {
  if (width == 0 || height == 0) return cudaSuccess;
  int sms = 0, ctas = 1;
  cudaError_t e = stageDevice(&sms, true, stream, &ctas);
  if (e != cudaSuccess) return e;
  PremulParams p;
  p.src = src;
  p.dst = dst;
  p.srcPitch = srcPitch;
  p.dstPitch = dstPitch;
  p.width = width;
  p.height = height;
  p.quadsPerRow = (width + 3) / 4;
  p.vec = (reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst) | srcPitch | dstPitch) % 16 == 0;
  const uint64_t quads = uint64_t(p.quadsPerRow) * height;
  const uint64_t perCta = uint64_t(kThreads) * kUnroll;
  // the resident CTAs (each holds a 64 KiB table copy), at most one pass over the image
  const uint32_t grid = uint32_t(std::min<uint64_t>((quads + perCta - 1) / perCta, uint64_t(sms) * ctas));
  premultiplyKernel<<<grid, kThreads, kSmemBytes, stream>>>(p);
  return cudaGetLastError();
}

}  // namespace nvpyr
