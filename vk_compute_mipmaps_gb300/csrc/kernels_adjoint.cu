// kernels_adjoint.cu -- adjoint (vector-Jacobian product) of the linear float
// pyramids (RGBA32F, RGBA16F storage with FP32 arithmetic).  No reference
// counterpart: the reference template admits float types
// (nvpro_pyramid.glsl:44-46) but ships no gradient.
//
// Forward: level k+1 = A_k level k, A_k separable with 1/2/3-tap weights
// (kernelSizeFromInputSize_, nvpro_pyramid.glsl:557-561; 3-tap weights
// :582-586).  For upstream gradients g_k on every level, the gradient of the
// base is h_0 with h_top = g_top and h_k = g_k + A_k^T h_{k+1}.  The sweep runs
// coarse to fine over the forward's dispatch schedule:
//  * a fast dispatch (L, n) has all 2x2 boxes, so every texel of level L has
//    one ancestor per level: h_L = g_L + 0.25 (g_{L+1} + 0.25 (... + 0.25
//    h_{L+n})).  One kernel evaluates that chain per texel and writes h_L once;
//    the coarse levels it reads are small and stay in cache;
//  * a general dispatch is handled level by level: each fine texel gathers
//    from its <= 2 parents per axis with the forward's FP32 weights.
// The operator is linear, so nothing of the forward pass is kept.
#include "device_common.cuh"

namespace nvpyr {

namespace {

// Storage types of gradient levels.
enum GradType : uint32_t { kF32 = 0, kF16 = 1 };

__device__ __forceinline__ float4 loadGrad(const uint8_t* base, uint64_t pitch, uint32_t type, uint32_t x,
                                           uint32_t y) {
  if (!base) return make_float4(0.f, 0.f, 0.f, 0.f);  // a level with no upstream gradient
  if (type == kF32) return *reinterpret_cast<const float4*>(base + y * pitch + uint64_t(x) * 16);
  const uint2 u = *reinterpret_cast<const uint2*>(base + y * pitch + uint64_t(x) * 8);
  const __half2 a = *reinterpret_cast<const __half2*>(&u.x);
  const __half2 b = *reinterpret_cast<const __half2*>(&u.y);
  return make_float4(__low2float(a), __high2float(a), __low2float(b), __high2float(b));
}

__device__ __forceinline__ void storeGrad(uint8_t* base, uint64_t pitch, uint32_t type, uint32_t x, uint32_t y,
                                          float4 v) {
  if (type == kF32) {
    *reinterpret_cast<float4*>(base + y * pitch + uint64_t(x) * 16) = v;
    return;
  }
  const __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
  uint2 u;
  u.x = *reinterpret_cast<const uint32_t*>(&a);
  u.y = *reinterpret_cast<const uint32_t*>(&b);
  *reinterpret_cast<uint2*>(base + y * pitch + uint64_t(x) * 8) = u;
}

// acc = g + s * h, as FMUL then FADD (each rounded once).
__device__ __forceinline__ float4 addScaled(float4 g, float s, float4 h) { return f4add(g, f4scale(s, h)); }

constexpr uint32_t kWarps = 8, kThreads = 32 * kWarps;

// Fast dispatch (L, n): h_L from h_{L+n} through the ancestor chain.  Lane =
// column of level L (a warp's loads and stores are 32 consecutive texels); each
// lane walks R rows (R = 4 if n >= 2, else 2) and shares the chain above level
// L + log2(R) between them.  Level sizes are multiples of 2^n, so R rows are
// always inside the level.
template <uint32_t R>
__global__ void __launch_bounds__(kThreads) adjointChainKernel(AdjointChainParams p) {
  constexpr uint32_t r = R == 4 ? 2 : 1;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t x = blockIdx.x * 32 + lane;
  if (x >= p.w) return;
  for (uint32_t y0 = (blockIdx.y * kWarps + warp) * R; y0 < p.h; y0 += gridDim.y * kWarps * R) {
    float4 v = loadGrad(p.top, p.topPitch, p.topType, x >> p.n, y0 >> p.n);
#pragma unroll
    for (int k = kMaxDispatchLevels - 1; k >= int(r); --k)
      if (k < int(p.n)) v = addScaled(loadGrad(p.g[k], p.gPitch[k], p.gType, x >> k, y0 >> k), 0.25f, v);
    float4 g0[R];
#pragma unroll
    for (uint32_t j = 0; j < R; ++j) g0[j] = loadGrad(p.g[0], p.gPitch[0], p.gType, x, y0 + j);
    if (R == 4) {
      const float4 a0 = addScaled(loadGrad(p.g[1], p.gPitch[1], p.gType, x >> 1, y0 >> 1), 0.25f, v);
      const float4 a1 = addScaled(loadGrad(p.g[1], p.gPitch[1], p.gType, x >> 1, (y0 >> 1) + 1), 0.25f, v);
#pragma unroll
      for (uint32_t j = 0; j < R; ++j)
        storeGrad(p.out, p.outPitch, p.outType, x, y0 + j, addScaled(g0[j], 0.25f, j < 2 ? a0 : a1));
    } else {
#pragma unroll
      for (uint32_t j = 0; j < R; ++j) storeGrad(p.out, p.outPitch, p.outType, x, y0 + j, addScaled(g0[j], 0.25f, v));
    }
  }
}

// Parents of fine coordinate i along one axis and their forward weights
// (count 1 or 2; unused entries have weight 0 and a valid index).
struct Parents {
  uint32_t count;
  uint32_t j[2];
  float w[2];
};

__device__ __forceinline__ Parents axisParents(uint32_t i, uint32_t fine, uint32_t coarse) {
  Parents r;
  r.j[1] = 0;
  r.w[1] = 0.0f;
  const uint32_t k = kernelSize(fine);
  if (k == 1) {
    r.count = 1;
    r.j[0] = 0;
    r.w[0] = 1.0f;
  } else if (k == 2) {
    r.count = 1;
    r.j[0] = i >> 1;
    r.w[0] = 0.5f;
  } else {
    // taps t = i - 2j in {0, 1, 2}, 0 <= j < coarse: j from ceil((i - 2) / 2)
    // to min(i / 2, coarse - 1)
    const uint32_t jHi = min(i >> 1, coarse - 1);
    const uint32_t jLo = i >= 2 ? (i - 1) >> 1 : 0;
    r.count = jHi - jLo + 1;
#pragma unroll
    for (uint32_t m = 0; m < 2; ++m) {
      if (m < r.count) {
        const uint32_t j = jLo + m;
        const Weights3 w = weights3(coarse, j);
        const uint32_t t = i - 2 * j;
        r.j[m] = j;
        r.w[m] = t == 0 ? w.w0 : t == 1 ? w.w1 : w.w2;
      }
    }
  }
  return r;
}

// One level of a general dispatch: h_k = g_k + A_k^T h_{k+1}.  Lane = column
// of level k (parents along x computed once); warps step over rows.
__global__ void __launch_bounds__(kThreads) adjointLevelKernel(AdjointLevelParams p) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t x = blockIdx.x * 32 + lane;
  if (x >= p.fw) return;
  const Parents px = axisParents(x, p.fw, p.cw);
  for (uint32_t y = blockIdx.y * kWarps + warp; y < p.fh; y += gridDim.y * kWarps) {
    const Parents py = axisParents(y, p.fh, p.ch);
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (uint32_t b = 0; b < 2; ++b) {
      if (b < py.count) {
        float4 s = addScaled(make_float4(0.f, 0.f, 0.f, 0.f), px.w[0],
                             loadGrad(p.hc, p.hcPitch, p.hcType, px.j[0], py.j[b]));
        if (px.count > 1) s = addScaled(s, px.w[1], loadGrad(p.hc, p.hcPitch, p.hcType, px.j[1], py.j[b]));
        t = addScaled(t, py.w[b], s);
      }
    }
    storeGrad(p.out, p.outPitch, p.outType, x, y, f4add(loadGrad(p.g, p.gPitch, p.gType, x, y), t));
  }
}

// 2D grid: one block column per 32 texel columns, enough block rows for
// about 32 blocks per SM, each warp stepping over `rowsPerWarp`-row strips.
dim3 gridFor(uint32_t w, uint32_t h, uint32_t rowsPerWarp) {
  const uint32_t gx = (w + 31) / 32;
  const uint32_t rowsNeeded = (h + kWarps * rowsPerWarp - 1) / (kWarps * rowsPerWarp);
  const uint32_t target = (152u * 32u + gx - 1) / gx;
  return dim3(gx, std::max(1u, std::min(rowsNeeded, target)));
}

}  // namespace

cudaError_t launchAdjointChain(const AdjointChainParams& p, cudaStream_t stream) {
  if (p.n >= 2)
    adjointChainKernel<4><<<gridFor(p.w, p.h, 4), kThreads, 0, stream>>>(p);
  else
    adjointChainKernel<2><<<gridFor(p.w, p.h, 2), kThreads, 0, stream>>>(p);
  return cudaGetLastError();
}

cudaError_t launchAdjointLevel(const AdjointLevelParams& p, cudaStream_t stream) {
  adjointLevelKernel<<<gridFor(p.fw, p.fh, 1), kThreads, 0, stream>>>(p);
  return cudaGetLastError();
}

}  // namespace nvpyr
