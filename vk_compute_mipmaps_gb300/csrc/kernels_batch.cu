// kernels_batch.cu -- many sRGBA8 images in one persistent launch.  No
// reference counterpart: the reference records one chain per command buffer
// (nvpro_pyramid_dispatch.hpp:109-188); its benchmark submits images one by
// one (demo_app/mipmaps_app.cpp:666-767).
//
// Phases.  Phase k runs the k-th dispatch of every image's default schedule
// (the dispatches of one image depend on each other, different images do
// not).  A bounded grid barrier separates phases, as the reference's pipeline
// barrier separates the dispatches of one chain.  The launch is cooperative
// (every CTA resident), so the barrier always completes; a wait that gives up
// after kWaitLimit polls sets the error flag and the kernel returns.
//
// Work queue.  Each phase is a list of jobs (one per image), sorted by size
// (largest first); a job is a run of units.  Warps take units from the
// phase's counter with one atomicAdd per unit, so images of any size mix
// without a tail of idle SMs.  Unit kinds:
//   fast  -- a 64x64 region of level L of a fast dispatch (fastRegion);
//   strip -- a general-pipeline strip (general_strip.cuh);
//   tiny  -- a whole general dispatch with a one-texel-wide level, done by
//            one warp texel by texel (tinyGeneral).
// Every unit computes its texels with the operation order of the per-image
// kernels, so the bytes equal a per-image nvproPyramidGenerate of each image.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "batch.h"
#include "general_strip.cuh"

namespace nvpyr {
namespace {

// CTA sizes the autotuner chooses from (WARPS template instances): 8 warps
// (up to 255 registers per thread) or 12 warps (168).
constexpr uint32_t kMaxWarps = 12;
constexpr uint32_t kRegion = 64;  // fast units: 64 texels of level L wide, `rows` high
constexpr uint32_t kTopBytes = kMaxDispatchLevels * 32 * 16;  // per warp: fast-region rows kept per level
constexpr uint32_t kJobIndexMax = 1024;  // jobs of a phase whose first units are searched in shared memory
template <uint32_t WARPS>
constexpr uint32_t kSmemBytesOf = kAlignedLutSmemBytes + WARPS * kTopBytes + kJobIndexMax * 4;
static_assert(kSmemBytesOf<kMaxWarps> + 1024 <= 232448, "exceeds the shared memory of a CTA");
constexpr uint32_t kFastGroupRows = 2;  // level-(L+1) rows of a fast region whose level-L rows load together
// Groups of rows a fast region asks L2 for beyond the group it holds in
// registers (prefetch.global.L2, as the strips do).
constexpr uint32_t kFastL2Groups = 2;

// One fast dispatch of n levels from level L (nvpro_pyramid.glsl:209-534).
struct FastJob {
  const uint8_t* src;
  uint64_t srcPitch;
  uint8_t* dst[kMaxDispatchLevels];
  uint64_t pitch[kMaxDispatchLevels];
  uint32_t n;
  uint32_t coverW, coverH;  // level L extent covered by whole 2^n tiles
  uint32_t regionsX;
  uint32_t rows;  // region height: a multiple of 2^n, at most kRegion
};

// A general dispatch with a one-texel-wide level (kernel size 1 on an axis).
struct TinyJob {
  const uint8_t* src;
  uint64_t srcPitch;
  uint8_t* dst[2];
  uint64_t pitch[2];
  uint32_t w[3], h[3];  // levels L, L+1, L+2
  uint32_t levels;
};

enum JobKind : uint32_t { kJobFast = 0, kJobStrip = 1, kJobTiny = 2 };

struct BatchJob {
  uint32_t kind;
  uint32_t unitBegin;  // first unit of the job in its phase
  uint32_t unitCount;
  uint32_t image;
  Stage strip;
  FastJob fast;
  TinyJob tiny;
};

struct BatchParams {
  const BatchJob* jobs;
  const uint32_t* phaseJobBegin;  // [phaseCount + 1]
  const uint32_t* phaseUnits;     // [phaseCount]
  uint32_t* unitCounters;         // [phaseCount], zero at launch
  uint32_t phaseCount;
  uint32_t* barrierCount;
  uint32_t* barrierGen;
  uint32_t* errorFlag;
};

__device__ __forceinline__ uint8_t* texel(uint8_t* base, uint64_t pitch, uint32_t x, uint32_t y) {
  return base + uint64_t(y) * pitch + uint64_t(x) * 4;
}

// One 64x64 region of a fast dispatch (rw x rh inside the covered extent,
// both multiples of 2^n).  Lane l holds level-L columns 2l, 2l+1 and walks
// the region's row pairs: level L+1 column l from its own 2x2 block
// (LOAD_REDUCE4, vertical pairs first); level L+k+1 from level L+k, whose
// values sit on lanes l = 0 mod 2^(k-1), pairing lane l with l + 2^(k-1)
// (shfl.down) and a row with the one kept from the previous odd step, in the
// operand order fastVerticalFirst(n, k+1).
__device__ __noinline__ void fastRegion(const FastJob& fjob, uint32_t unit, uint32_t lane, const Lut& L,
                                        float4* top) {
  // The fields of every row in registers (stores cannot force their
  // reloads); the deeper levels' views are read from the job when stored.
  const FastJob& f = fjob;
  const uint32_t n = f.n, regionsX = f.regionsX, coverW = f.coverW, coverH = f.coverH;
  const uint64_t pitch = f.srcPitch;
  const uint8_t* const src = f.src;
  uint8_t* const d1 = f.dst[0];
  const uint64_t p1 = f.pitch[0];
  const uint32_t x0 = (unit % regionsX) * kRegion, y0 = (unit / regionsX) * f.rows;
  const uint32_t rw = min(kRegion, coverW - x0), rh = min(f.rows, coverH - y0);
  const bool colOk = 2 * lane < rw;
  const uint8_t* base = src + uint64_t(y0) * pitch + uint64_t(x0 + (colOk ? 2 * lane : 0)) * 4;
  const uint32_t rows1 = rh / 2;  // level-(L+1) rows of the region

  auto ldGroup = [&](uint32_t r0, uint32_t (&raw)[kFastGroupRows][4]) {
    const uint8_t* row = base + uint64_t(2 * r0) * pitch;
#pragma unroll
    for (uint32_t j = 0; j < kFastGroupRows; ++j) {
      if (r0 + j < rows1) {
        raw[j][0] = ldTexel(row);              // (2l,   y)
        raw[j][1] = ldTexel(row + 4);          // (2l+1, y)
        raw[j][2] = ldTexel(row + pitch);      // (2l,   y+1)
        raw[j][3] = ldTexel(row + pitch + 4);  // (2l+1, y+1)
      }
      row += 2 * pitch;
    }
  };

  auto pfGroup = [&](uint32_t r0) {  // ask L2 for the level-L rows of group r0
    const uint8_t* row = base + uint64_t(2 * r0) * pitch;
#pragma unroll
    for (uint32_t j = 0; j < kFastGroupRows; ++j) {
      if (r0 + j < rows1) {
        prefetchL2(row);
        prefetchL2(row + pitch);
      }
      row += 2 * pitch;
    }
  };

  // top[32 k + lane]: level k's row kept from its last even step (the
  // warp's slice of shared memory)
  auto process = [&](uint32_t r0, const uint32_t (&raw)[kFastGroupRows][4]) {
#pragma unroll
    for (uint32_t j = 0; j < kFastGroupRows; ++j) {
      const uint32_t r = r0 + j;
      if (r >= rows1) break;
      float4 v = reduce4p(decodeAligned(raw[j][0], L), decodeAligned(raw[j][2], L), decodeAligned(raw[j][1], L),
                          decodeAligned(raw[j][3], L));
      if (colOk) *reinterpret_cast<uint32_t*>(texel(d1, p1, (x0 >> 1) + lane, (y0 >> 1) + r)) = encodeTexel(v, L);
      uint32_t rk = r;
#pragma unroll 1
      for (uint32_t k = 1; k < n; ++k) {
        if ((rk & 1) == 0) {
          top[32 * k + lane] = v;
          break;
        }
        const float4 t = top[32 * k + lane];
        const uint32_t s = 1u << (k - 1);
        const float4 tr = shflDown(t, s), br = shflDown(v, s);
        v = fastVerticalFirst(n, k + 1) ? reduce4p(t, v, tr, br) : reduce4p(t, tr, v, br);
        rk >>= 1;
        const uint32_t col = lane >> k;
        if ((lane & (2 * s - 1)) == 0 && col < (rw >> (k + 1)))
          *reinterpret_cast<uint32_t*>(texel(f.dst[k], f.pitch[k], (x0 >> (k + 1)) + col, (y0 >> (k + 1)) + rk)) =
              encodeTexel(v, L);
      }
    }
  };

  uint32_t bufA[kFastGroupRows][4], bufB[kFastGroupRows][4];
  ldGroup(0, bufA);
  constexpr uint32_t kPf = kFastGroupRows * (kFastL2Groups + 1);  // rows ahead of r0 asked of L2
#pragma unroll
  for (uint32_t g = 2; g <= kFastL2Groups; ++g) pfGroup(g * kFastGroupRows);
  for (uint32_t r0 = 0;;) {
    if (r0 + kFastGroupRows < rows1) ldGroup(r0 + kFastGroupRows, bufB);
    if (kFastL2Groups && r0 + kPf < rows1) pfGroup(r0 + kPf);
    process(r0, bufA);
    r0 += kFastGroupRows;
    if (r0 >= rows1) break;
    if (r0 + kFastGroupRows < rows1) ldGroup(r0 + kFastGroupRows, bufA);
    if (kFastL2Groups && r0 + kPf < rows1) pfGroup(r0 + kPf);
    process(r0, bufB);
    r0 += kFastGroupRows;
    if (r0 >= rows1) break;
  }
}

// One output texel of the general kernel (reduceStoreSample_,
// nvpro_pyramid.glsl:575-656): kernel sizes kx, ky from the input size,
// vertical reductions per column first, `ld(dx, dy)` the FP32 input at
// (2x + dx, 2y + dy).
template <typename Load>
__device__ __forceinline__ float4 sampleAt(const Load& ld, uint32_t kx, uint32_t ky, uint32_t dstW, uint32_t dstH,
                                           uint32_t x, uint32_t y) {
  float4 h[3];
#pragma unroll
  for (uint32_t c = 0; c < 3; ++c) {
    if (c >= kx) break;
    if (ky == 3)
      h[c] = reduce3(weights3(dstH, y).w0, ld(c, 0), weights3(dstH, y).w1, ld(c, 1), weights3(dstH, y).w2, ld(c, 2));
    else if (ky == 2)
      h[c] = reduce2(ld(c, 0), ld(c, 1));
    else
      h[c] = ld(c, 0);
  }
  if (kx == 3) {
    const Weights3 wx = weights3(dstW, x);
    return reduce3(wx.w0, h[0], wx.w1, h[1], wx.w2, h[2]);
  }
  if (kx == 2) return reduce2(h[0], h[1]);
  return h[0];
}

// A whole general dispatch with a one-texel-wide level, by one warp: lanes
// take level-(L+1) texels in turn; for level L+2 each texel recomputes the
// FP32 level-(L+1) values it reads (the same values, in the same order).
__device__ __noinline__ void tinyGeneral(const TinyJob& tj, uint32_t lane, const Lut& L) {
  const TinyJob t = tj;
  const uint32_t kx0 = kernelSize(t.w[0]), ky0 = kernelSize(t.h[0]);
  auto l0 = [&](uint32_t x, uint32_t y) { return decodeAligned(ldTexel(t.src + uint64_t(y) * t.srcPitch + uint64_t(x) * 4), L); };
  auto l1 = [&](uint32_t x, uint32_t y) {
    auto ld = [&](uint32_t dx, uint32_t dy) { return l0(2 * x + dx, 2 * y + dy); };
    return sampleAt(ld, kx0, ky0, t.w[1], t.h[1], x, y);
  };
  const uint32_t n1 = t.w[1] * t.h[1];
  for (uint32_t i = lane; i < n1; i += 32) {
    const uint32_t x = i % t.w[1], y = i / t.w[1];
    *reinterpret_cast<uint32_t*>(texel(t.dst[0], t.pitch[0], x, y)) = encodeTexel(l1(x, y), L);
  }
  if (t.levels < 2) return;
  const uint32_t kx1 = kernelSize(t.w[1]), ky1 = kernelSize(t.h[1]);
  const uint32_t n2 = t.w[2] * t.h[2];
  for (uint32_t i = lane; i < n2; i += 32) {
    const uint32_t x = i % t.w[2], y = i / t.w[2];
    auto ld = [&](uint32_t dx, uint32_t dy) { return l1(2 * x + dx, 2 * y + dy); };
    *reinterpret_cast<uint32_t*>(texel(t.dst[1], t.pitch[1], x, y)) =
        encodeTexel(sampleAt(ld, kx1, ky1, t.w[2], t.h[2], x, y), L);
  }
}

// Out of line, each unit kind gets its own register allocation; the call
// costs a few register saves per unit.
__device__ __noinline__ void stripUnit(const Stage& st, uint32_t local, uint32_t lane, const Lut& L) {
  strip<kSharedFp32>(st, local % st.tilesX, local / st.tilesX, lane, L);
}

template <uint32_t WARPS>
__global__ void __launch_bounds__(32 * WARPS, 1) batchKernel(const __grid_constant__ BatchParams p) {
  constexpr uint32_t kWarps = WARPS, kThreads = 32 * WARPS;
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint32_t okFlag;
  const Lut L = fillAlignedLut<(768 + kThreads - 1) / kThreads>(smem, threadIdx.x, kThreads);
  uint32_t gen = 0;
  if (threadIdx.x == 0 && p.phaseCount > 1) gen = ldAcquire(p.barrierGen);  // before this CTA's first arrival
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  float4* const top = reinterpret_cast<float4*>(smem + kAlignedLutSmemBytes + (threadIdx.x >> 5) * kTopBytes);
  // first unit of each job of the current phase (the unit -> job search)
  uint32_t* const jobStart = reinterpret_cast<uint32_t*>(smem + kAlignedLutSmemBytes + kWarps * kTopBytes);
#pragma unroll 1
  for (uint32_t k = 0; k < p.phaseCount; ++k) {
    const uint32_t jb = p.phaseJobBegin[k], je = p.phaseJobBegin[k + 1], units = p.phaseUnits[k];
    const bool inSmem = je - jb <= kJobIndexMax;
    if (inSmem)
      for (uint32_t j = threadIdx.x; j < je - jb; j += kThreads) jobStart[j] = p.jobs[jb + j].unitBegin;
    __syncthreads();
    for (;;) {
      uint32_t u = 0;
      if (lane == 0) u = atomicAdd(p.unitCounters + k, 1u);
      u = __shfl_sync(0xffffffffu, u, 0);
      if (u >= units) break;
      uint32_t lo = jb, hi = je - 1;  // the last job of the phase with unitBegin <= u
      while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if ((inSmem ? jobStart[mid - jb] : p.jobs[mid].unitBegin) <= u) lo = mid;
        else hi = mid - 1;
      }
      const BatchJob& J = p.jobs[lo];
      const uint32_t local = u - J.unitBegin;
      if (J.kind == kJobFast)
        fastRegion(J.fast, local, lane, L, top);
      else if (J.kind == kJobStrip)
        stripUnit(J.strip, local, lane, L);
      else
        tinyGeneral(J.tiny, lane, L);
    }
    if (k + 1 < p.phaseCount && !gridBarrierWait(p.barrierCount, p.barrierGen, p.errorFlag, gen, &okFlag)) return;
  }
}

struct DeviceState {
  int sms = 0;
};

template <uint32_t WARPS>
cudaError_t setUp(int dev) {
  cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(batchKernel<WARPS>),
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemBytesOf<WARPS>));
  int ctasPerSm = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctasPerSm, batchKernel<WARPS>, 32 * WARPS,
                                                      kSmemBytesOf<WARPS>);
  if (e == cudaSuccess && ctasPerSm < 1) e = cudaErrorInvalidConfiguration;
  return e;
}

cudaError_t deviceState(int* sms) {
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
    e = setUp<8>(dev);
    if (e == cudaSuccess) e = setUp<12>(dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  *sms = d.sms;
  return cudaSuccess;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side: plan and launch.

struct BatchPlan::Tables {
  std::vector<BatchJob> jobs;
  std::vector<uint32_t> phaseJobBegin;
  std::vector<uint32_t> phaseUnits;
};

BatchPlan::BatchPlan() : t_(new Tables) {}
BatchPlan::~BatchPlan() { delete t_; }

uint32_t BatchPlan::phaseCount() const { return uint32_t(t_->phaseUnits.size()); }
uint32_t BatchPlan::jobCount() const { return uint32_t(t_->jobs.size()); }
uint64_t BatchPlan::unitCount() const {
  uint64_t u = 0;
  for (uint32_t x : t_->phaseUnits) u += x;
  return u;
}

uint64_t BatchPlan::deviceBytes() const {
  const uint64_t phases = t_->phaseUnits.size();
  return t_->jobs.size() * sizeof(BatchJob) + (2 * phases + 1) * 4 + phases * 4 + 4 * 4 + 256;
}

cudaError_t BatchPlan::build(const std::vector<std::vector<DispatchParams>>& images, const BatchTuning& tuning) {
  const uint32_t stripBand = tuning.stripBand;
  Tables& t = *t_;
  t.jobs.clear();
  t.phaseJobBegin.assign(1, 0);
  t.phaseUnits.clear();
  size_t phases = 0;
  for (const auto& img : images) phases = std::max(phases, img.size());
  for (size_t k = 0; k < phases; ++k) {
    std::vector<std::pair<uint64_t, BatchJob>> jobs;  // (input texels, job)
    for (uint32_t i = 0; i < images.size(); ++i) {
      if (k >= images[i].size()) continue;
      const DispatchParams& d = images[i][k];
      if (d.preset != kSrgba8) return cudaErrorInvalidValue;
      BatchJob j{};
      j.image = i;
      if (d.isFast) {
        const uint32_t n = d.levelCount;
        const uint32_t cw = (d.lv[0].w >> n) << n, ch = (d.lv[0].h >> n) << n;
        // the default dispatcher covers every tile (nvproPyramidDefaultFastDispatcher)
        const uint64_t tiles = uint64_t(d.lv[0].w >> n) * (d.lv[0].h >> n);
        const uint64_t perGroup = std::max<uint64_t>(1, (n > 5 ? 4096u : 1024u) >> (2 * n));
        if (d.groups * perGroup < tiles || cw == 0 || ch == 0) return cudaErrorInvalidValue;
        j.kind = kJobFast;
        j.fast.src = d.lv[0].ptr;
        j.fast.srcPitch = d.lv[0].pitch;
        for (uint32_t l = 0; l < n; ++l) {
          j.fast.dst[l] = d.lv[l + 1].ptr;
          j.fast.pitch[l] = d.lv[l + 1].pitch;
        }
        j.fast.n = n;
        j.fast.coverW = cw;
        j.fast.coverH = ch;
        j.fast.regionsX = (cw + kRegion - 1) / kRegion;
        j.fast.rows = std::min(kRegion, std::max(tuning.fastRows, 1u << n));  // whole 2^n tiles per region
        j.unitCount = j.fast.regionsX * ((ch + j.fast.rows - 1) / j.fast.rows);
      } else if (generalFastSupported(d)) {
        j.kind = kJobStrip;
        stageGeometry(d, &j.strip);
        setStageBand(&j.strip, d.levelCount == 2 ? stripBand : 2 * stripBand);
        j.unitCount = j.strip.tilesX * j.strip.bands;
      } else {
        // a one-texel-wide level; the default dispatcher covers everything
        j.kind = kJobTiny;
        j.tiny.src = d.lv[0].ptr;
        j.tiny.srcPitch = d.lv[0].pitch;
        j.tiny.levels = d.levelCount;
        for (uint32_t l = 0; l <= d.levelCount; ++l) {
          j.tiny.w[l] = d.lv[l].w;
          j.tiny.h[l] = d.lv[l].h;
          if (l > 0) {
            j.tiny.dst[l - 1] = d.lv[l].ptr;
            j.tiny.pitch[l - 1] = d.lv[l].pitch;
          }
        }
        if (d.levelCount == 1) j.tiny.w[2] = j.tiny.h[2] = 1;
        j.unitCount = 1;
      }
      jobs.emplace_back(uint64_t(d.lv[0].w) * d.lv[0].h, j);
    }
    // largest first: big jobs' units are taken first, small ones fill the tail
    std::stable_sort(jobs.begin(), jobs.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    uint32_t units = 0;
    for (auto& pj : jobs) {
      pj.second.unitBegin = units;
      units += pj.second.unitCount;
      t.jobs.push_back(pj.second);
    }
    t.phaseJobBegin.push_back(uint32_t(t.jobs.size()));
    t.phaseUnits.push_back(units);
  }
  return cudaSuccess;
}

// Device block layout: jobs | phaseJobBegin | phaseUnits | unitCounters | barrier words.
cudaError_t BatchPlan::upload(void* device, cudaStream_t stream, BatchDevice* out) const {
  const Tables& t = *t_;
  const uint64_t phases = t.phaseUnits.size();
  std::vector<uint8_t> host(deviceBytes(), 0);
  uint64_t off = 0;
  auto put = [&](const void* src, uint64_t bytes) {
    std::memcpy(host.data() + off, src, bytes);
    const uint64_t at = off;
    off += (bytes + 15) & ~uint64_t(15);
    return at;
  };
  const uint64_t jobsOff = put(t.jobs.data(), t.jobs.size() * sizeof(BatchJob));
  const uint64_t beginOff = put(t.phaseJobBegin.data(), t.phaseJobBegin.size() * 4);
  const uint64_t unitsOff = put(t.phaseUnits.data(), phases * 4);
  out->countersOffset = off;
  out->countersBytes = phases * 4 + 3 * 4;  // unit counters, barrier count, generation, error flag
  off += (out->countersBytes + 15) & ~uint64_t(15);
  if (off > host.size()) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemcpyAsync(device, host.data(), off, cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(stream);  // `host` goes out of scope
  if (e != cudaSuccess) return e;
  uint8_t* base = static_cast<uint8_t*>(device);
  out->device = device;
  out->jobs = base + jobsOff;
  out->phaseJobBegin = reinterpret_cast<uint32_t*>(base + beginOff);
  out->phaseUnits = reinterpret_cast<uint32_t*>(base + unitsOff);
  out->counters = reinterpret_cast<uint32_t*>(base + out->countersOffset);
  out->phaseCount = uint32_t(phases);
  return cudaSuccess;
}

uint64_t BatchPlan::errorFlagOffset() const { return phaseCount() * 4 + 8; }

cudaError_t batchDeviceReady() {
  int sms = 0;
  return deviceState(&sms);
}

cudaError_t launchBatch(const BatchDevice& d, cudaStream_t stream, uint32_t* launches) {
  if (d.phaseCount == 0) return cudaSuccess;
  if (d.warps != 8 && d.warps != 12) return cudaErrorInvalidValue;
  int sms = 0;
  cudaError_t e = deviceState(&sms);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(d.counters, 0, d.phaseCount * 4 + 8, stream);  // unit counters and barrier count
  if (e != cudaSuccess) return e;
  BatchParams p{};
  p.jobs = static_cast<const BatchJob*>(d.jobs);
  p.phaseJobBegin = d.phaseJobBegin;
  p.phaseUnits = d.phaseUnits;
  p.unitCounters = d.counters;
  p.phaseCount = d.phaseCount;
  p.barrierCount = d.counters + d.phaseCount;
  p.barrierGen = d.counters + d.phaseCount + 1;
  p.errorFlag = d.counters + d.phaseCount + 2;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(uint32_t(sms));  // one CTA per SM (all resident: the phases' grid barriers)
  cfg.blockDim = dim3(32 * d.warps);
  cfg.dynamicSmemBytes = d.warps == 8 ? kSmemBytesOf<8> : kSmemBytesOf<12>;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = d.warps == 8 ? cudaLaunchKernelEx(&cfg, batchKernel<8>, p) : cudaLaunchKernelEx(&cfg, batchKernel<12>, p);
  if (e != cudaSuccess) return e;
  ++*launches;
  return cudaSuccess;
}

}  // namespace nvpyr
