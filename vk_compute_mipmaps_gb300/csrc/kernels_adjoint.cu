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

// A texel of zeros: levels without an upstream gradient read it with row pitch
// and texel stride 0, so every load of the kernels below is unconditional.
__device__ __align__(16) float g_zeroTexel[4];

// Gradient storage: FP32 (16 bytes per texel) or FP16 (8 bytes per texel).
template <bool F16>
struct Grad {
  static constexpr uint32_t kBytes = F16 ? 8 : 16;
  __device__ static __forceinline__ float4 load(const uint8_t* p) {
    if (!F16) return *reinterpret_cast<const float4*>(p);
    const uint2 u = *reinterpret_cast<const uint2*>(p);
    const __half2 a = *reinterpret_cast<const __half2*>(&u.x);
    const __half2 b = *reinterpret_cast<const __half2*>(&u.y);
    return make_float4(__low2float(a), __high2float(a), __low2float(b), __high2float(b));
  }
  __device__ static __forceinline__ void store(uint8_t* p, float4 v) {
    if (!F16) {
      *reinterpret_cast<float4*>(p) = v;
      return;
    }
    const __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
    uint2 u;
    u.x = *reinterpret_cast<const uint32_t*>(&a);
    u.y = *reinterpret_cast<const uint32_t*>(&b);
    *reinterpret_cast<uint2*>(p) = u;
  }
};

// Read view of one level: address of texel (x, y) = base + y * pitch + x * stride.
struct View {
  const uint8_t* base;
  uint64_t pitch;
  uint32_t stride;
  __device__ __forceinline__ const uint8_t* at(uint32_t x, uint32_t y) const {
    return base + uint64_t(y) * pitch + uint64_t(x) * stride;
  }
};

// The view of image blockIdx.z of a level (image stride `image` bytes).
template <bool F16>
__device__ __forceinline__ View viewOf(const uint8_t* p, uint64_t pitch, uint64_t image) {
  if (p) return View{p + uint64_t(blockIdx.z) * image, pitch, Grad<F16>::kBytes};
  return View{reinterpret_cast<const uint8_t*>(g_zeroTexel), 0, 0};
}

// acc = g + s * h, as FMUL then FADD (each rounded once).
__device__ __forceinline__ float4 addScaled(float4 g, float s, float4 h) { return f4add(g, f4scale(s, h)); }

constexpr uint32_t kWarps = 8, kThreads = 32 * kWarps;

// Fast dispatch (L, n): h_L from h_{L+n} through the ancestor chain.  Lane =
// column of level L (a warp's loads and stores are 32 consecutive texels); each
// lane walks 2^LR rows (LR = min(n, 3)) and shares the chain above level L + LR
// between them, expanding it one level at a time (rows double per level).
// Level sizes are multiples of 2^n, so the rows are always inside the level.
// GF16 / TF16 / OF16: FP16 storage of the upstream gradients / of h_{L+n} /
// of h_L (else FP32).
template <uint32_t LR, bool GF16, bool TF16, bool OF16>
__global__ void __launch_bounds__(kThreads) adjointChainKernel(AdjointChainParams p) {
  constexpr uint32_t R = 1u << LR;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t x = blockIdx.x * 32 + lane;
  if (x >= p.w) return;
  const uint32_t n = p.n;
  const View top = viewOf<TF16>(p.top, p.topPitch, p.topImage);
  View g[kMaxDispatchLevels];
#pragma unroll
  for (uint32_t k = 0; k < kMaxDispatchLevels; ++k)
    g[k] = viewOf<GF16>(k < n ? p.g[k] : nullptr, p.gPitch[k], p.gImage[k]);
  uint8_t* const out = p.out + uint64_t(blockIdx.z) * p.outImage;
  for (uint32_t y0 = (blockIdx.y * kWarps + warp) * R; y0 < p.h; y0 += gridDim.y * kWarps * R) {
    // every load of the strip first, then the arithmetic
    const float4 t = Grad<TF16>::load(top.at(x >> n, y0 >> n));
    float4 c[kMaxDispatchLevels];
#pragma unroll
    for (int k = kMaxDispatchLevels - 1; k >= int(LR); --k) c[k] = Grad<GF16>::load(g[k].at(x >> k, y0 >> k));
    float4 rows[2 * R];  // level L + k, k < LR: 2^(LR - k) rows at offset 2^(LR - k) - 2
#pragma unroll
    for (int k = int(LR) - 1; k >= 0; --k) {
      const uint32_t cnt = 1u << (LR - k);
#pragma unroll
      for (uint32_t j = 0; j < cnt; ++j) rows[cnt - 2 + j] = Grad<GF16>::load(g[k].at(x >> k, (y0 >> k) + j));
    }
    float4 cur[R];
    cur[0] = t;
#pragma unroll
    for (int k = kMaxDispatchLevels - 1; k >= int(LR); --k)
      if (k < int(n)) cur[0] = addScaled(c[k], 0.25f, cur[0]);
#pragma unroll
    for (int k = int(LR) - 1; k >= 0; --k) {
      const uint32_t cnt = 1u << (LR - k);
#pragma unroll
      for (int j = int(cnt) - 1; j >= 0; --j) cur[j] = addScaled(rows[cnt - 2 + j], 0.25f, cur[j >> 1]);
    }
#pragma unroll
    for (uint32_t j = 0; j < R; ++j)
      Grad<OF16>::store(out + uint64_t(y0 + j) * p.outPitch + uint64_t(x) * Grad<OF16>::kBytes, cur[j]);
  }
}

// Parents of fine coordinate i along one axis and their forward weights
// (count 1 or 2; an unused second entry has weight 0 and index 0).
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
template <bool GF16, bool CF16, bool OF16>
__global__ void __launch_bounds__(kThreads) adjointLevelKernel(AdjointLevelParams p) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t x = blockIdx.x * 32 + lane;
  if (x >= p.fw) return;
  const View g = viewOf<GF16>(p.g, p.gPitch, p.gImage);
  const View hc = viewOf<CF16>(p.hc, p.hcPitch, p.hcImage);
  uint8_t* const out = p.out + uint64_t(blockIdx.z) * p.outImage;
  const Parents px = axisParents(x, p.fw, p.cw);
  for (uint32_t y = blockIdx.y * kWarps + warp; y < p.fh; y += gridDim.y * kWarps) {
    const Parents py = axisParents(y, p.fh, p.ch);
    // the second parent of an axis with one parent has weight 0 and index 0:
    // loading it is harmless, and skipping it keeps the FP32 order of a sum
    // over the actual parents
    float4 v[2][2];
#pragma unroll
    for (uint32_t b = 0; b < 2; ++b)
#pragma unroll
      for (uint32_t a = 0; a < 2; ++a) v[b][a] = Grad<CF16>::load(hc.at(px.j[a], py.j[b]));
    const float4 gk = Grad<GF16>::load(g.at(x, y));
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (uint32_t b = 0; b < 2; ++b) {
      if (b < py.count) {
        float4 s = addScaled(make_float4(0.f, 0.f, 0.f, 0.f), px.w[0], v[b][0]);
        if (px.count > 1) s = addScaled(s, px.w[1], v[b][1]);
        t = addScaled(t, py.w[b], s);
      }
    }
    Grad<OF16>::store(out + uint64_t(y) * p.outPitch + uint64_t(x) * Grad<OF16>::kBytes, f4add(gk, t));
  }
}

// 2D grid: one block column per 32 texel columns, enough block rows for
// about 32 blocks per SM, each warp stepping over `rowsPerWarp`-row strips.
dim3 gridFor(uint32_t w, uint32_t h, uint32_t rowsPerWarp, uint32_t batch) {
  const uint32_t gx = (w + 31) / 32;
  const uint32_t rowsNeeded = (h + kWarps * rowsPerWarp - 1) / (kWarps * rowsPerWarp);
  const uint32_t target = (152u * 32u + gx * batch - 1) / (gx * batch);
  return dim3(gx, std::max(1u, std::min(rowsNeeded, target)), batch);
}

template <uint32_t LR, bool GF16>
void launchChain(const AdjointChainParams& p, cudaStream_t s) {
  const dim3 grid = gridFor(p.w, p.h, 1u << LR, p.batch);
  const uint32_t sel = (p.topType ? 2u : 0u) | (p.outType ? 1u : 0u);
  switch (sel) {
    case 0: adjointChainKernel<LR, GF16, false, false><<<grid, kThreads, 0, s>>>(p); break;
    case 1: adjointChainKernel<LR, GF16, false, true><<<grid, kThreads, 0, s>>>(p); break;
    case 2: adjointChainKernel<LR, GF16, true, false><<<grid, kThreads, 0, s>>>(p); break;
    default: adjointChainKernel<LR, GF16, true, true><<<grid, kThreads, 0, s>>>(p); break;
  }
}

template <bool GF16>
void launchLevel(const AdjointLevelParams& p, cudaStream_t s) {
  const dim3 grid = gridFor(p.fw, p.fh, 1, p.batch);
  const uint32_t sel = (p.hcType ? 2u : 0u) | (p.outType ? 1u : 0u);
  switch (sel) {
    case 0: adjointLevelKernel<GF16, false, false><<<grid, kThreads, 0, s>>>(p); break;
    case 1: adjointLevelKernel<GF16, false, true><<<grid, kThreads, 0, s>>>(p); break;
    case 2: adjointLevelKernel<GF16, true, false><<<grid, kThreads, 0, s>>>(p); break;
    default: adjointLevelKernel<GF16, true, true><<<grid, kThreads, 0, s>>>(p); break;
  }
}

}  // namespace

cudaError_t launchAdjointChain(const AdjointChainParams& p, cudaStream_t stream) {
  const bool f16 = p.gType != 0;
  if (p.n >= 3)
    f16 ? launchChain<3, true>(p, stream) : launchChain<3, false>(p, stream);
  else if (p.n == 2)
    f16 ? launchChain<2, true>(p, stream) : launchChain<2, false>(p, stream);
  else
    f16 ? launchChain<1, true>(p, stream) : launchChain<1, false>(p, stream);
  return cudaGetLastError();
}

cudaError_t launchAdjointLevel(const AdjointLevelParams& p, cudaStream_t stream) {
  p.gType ? launchLevel<true>(p, stream) : launchLevel<false>(p, stream);
  return cudaGetLastError();
}

}  // namespace nvpyr
