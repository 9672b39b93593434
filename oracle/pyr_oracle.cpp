// pyr_oracle.cpp -- CPU ORACLE FOR TESTS ONLY.
//
// This file is test infrastructure: a scalar C++ restatement of the reference
// nvpro_pyramid mip-chain generation, the oracle that tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg compare against.  No
// product code path calls it.  Build: make -C oracle (g++ -O2
// -ffp-contract=off).
//
// Parity pins (see tests/test_oracle_pins.py):
//  * orc_refcpu_srgba8 restates the reference's own CPU generator
//    (include/mipmap_storage.hpp:204-414) and is checked bit-exact against it
//    (compiled from the reference sources into oracle/_ref/ where the sources
//    exist, and against committed golden vectors made that way otherwise).
//  * orc_default_schedule restates nvpro_pyramid_dispatch.hpp:109-304 and is
//    checked against the reference header itself compiled with a recording
//    Vulkan stub (golden dispatch sequences).
//  * orc_run restates the shader arithmetic (nvpro_pyramid.glsl,
//    srgba8_mipmap_preamble.glsl) dispatch by dispatch.  The reference shaders
//    cannot run here (no graphics stack), so this mode is pinned only through
//    the worst-delta bar against the reference CPU generator (the reference's
//    own bar: demo_app/rtx3090.json reports delta 2 on opaque images).
//
// Implementation-defined points of the reference shaders are pinned as follows
// (GPU and oracle agree bit for bit on these choices):
//  * no FMA contraction: every multiply and add rounds separately, as written;
//  * divisions (1.0f / (2n+1)) are IEEE correctly rounded;
//  * sRGB decode is the FP32 nearest to the exact EOTF (texelFetch of an SRGB
//    format, preamble.glsl:21-22); alpha decode is the FP32 nearest to c/255;
//  * sRGB encode is the exact OETF rounded as srgbFromLinearBias(x, 0.5)
//    (preamble.glsl:110-121) would with exact arithmetic;
//  * LOAD_REDUCE4 is the four-texelFetch form (nvpro_pyramid.glsl:180-188),
//    not the bilinear textureLod form (preamble.glsl:40-58), whose filter
//    precision is hardware-defined.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Vec4 {
  float v[4];
};

// --------------------------------------------------------------------------
// sRGB tables, computed here independently of the library's generated header
// (long double arithmetic; the tests compare both).

struct SrgbTables {
  float decode[256];
  float alpha[256];
  float thr[256];  // thr[a] = smallest x with code(x) >= a + 1; thr[255] = +inf
  SrgbTables() {
    for (int c = 0; c < 256; ++c) {
      long double u = (long double)c / 255.0L;
      long double lin = u <= 0.04045L ? u / 12.92L : powl((u + 0.055L) / 1.055L, 2.4L);
      decode[c] = (float)lin;
      alpha[c] = (float)c / 255.0f;  // IEEE single division: correctly rounded
    }
    for (int a = 0; a < 255; ++a) {
      const long double target = ((long double)a + 0.5L) / 255.0L;
      uint32_t lo = 0, hi = 0x3F800000u;  // 0.0f .. 1.0f
      while (hi - lo > 1) {
        uint32_t mid = lo + (hi - lo) / 2;
        float x;
        std::memcpy(&x, &mid, 4);
        if (oetf(x) >= target)
          hi = mid;
        else
          lo = mid;
      }
      std::memcpy(&thr[a], &hi, 4);
    }
    thr[255] = INFINITY;
  }
  static long double oetf(float xf) {
    long double x = xf;
    return x <= 0.0031308L ? 12.92L * x : 1.055L * powl(x, 5.0L / 12.0L) - 0.055L;
  }
};

const SrgbTables& tables() {
  static SrgbTables t;
  return t;
}

uint32_t srgbEncode(float x) {
  // Number of thresholds <= x (0 for NaN).
  const float* t = tables().thr;
  uint32_t n = 0;
  for (int step = 128; step > 0; step >>= 1)
    if (n + step <= 255 && t[n + step - 1] <= x) n += step;
  return n;
}

uint32_t alphaEncode(float a) {
  // srgba8_mipmap_preamble.glsl:125: clamp(uint(a * 255.0f + 0.5f), 0u, 255u)
  float s = a * 255.0f;
  s = s + 0.5f;
  if (!(s >= 0.0f)) return 0;
  if (s >= 256.0f) return 255;
  uint32_t q = (uint32_t)s;
  return q > 255 ? 255 : q;
}

// IEEE binary16 <-> binary32, round to nearest even.
float halfToFloat(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t exp = (h >> 10) & 0x1Fu;
  uint32_t man = h & 0x3FFu;
  uint32_t bits;
  if (exp == 0) {
    if (man == 0) {
      bits = sign;
    } else {  // subnormal: value = man * 2^-24
      float f = (float)man * (1.0f / 16777216.0f);
      std::memcpy(&bits, &f, 4);
      bits |= sign;
    }
  } else if (exp == 31) {
    bits = sign | 0x7F800000u | (man << 13);
  } else {
    bits = sign | ((exp + 112u) << 23) | (man << 13);
  }
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}

uint16_t floatToHalf(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  uint16_t sign = (uint16_t)((x >> 16) & 0x8000u);
  uint32_t ax = x & 0x7FFFFFFFu;
  if (ax >= 0x7F800000u) return (uint16_t)(sign | 0x7C00u | (ax > 0x7F800000u ? 0x200u : 0u));
  if (ax >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);  // rounds to >= 65520 -> inf
  if (ax < 0x38800000u) {  // below 2^-14: subnormal half (or zero)
    // value * 2^24 rounded to nearest even integer = subnormal mantissa
    float a;
    std::memcpy(&a, &ax, 4);
    double scaled = (double)a * 16777216.0;  // exact
    double r = std::nearbyint(scaled);       // default rounding mode: to nearest even
    return (uint16_t)(sign | (uint16_t)r);
  }
  uint32_t exp = (ax >> 23) - 112u;
  uint32_t man = ax & 0x7FFFFFu;
  uint32_t h = (exp << 10) | (man >> 13);
  uint32_t rem = man & 0x1FFFu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h += 1;  // carries into exponent correctly
  return (uint16_t)(sign | h);
}

// --------------------------------------------------------------------------
// Images in the packed MipmapStorage layout (include/mipmap_storage.hpp:53-76).

// kRgba16Unorm is no preset of the library: the texel format of the custom
// functor set the tests compile against nvpro_pyramid_cuda.hpp (RGBA 16-bit
// unorm, load c / 65535, store uint(clamp(v, 0, 1) * 65535 + 0.5)), which
// defines REDUCE only, so its REDUCE2 and REDUCE4 are the reference's defaults
// (nvpro_pyramid.glsl:164-177): REDUCE(0.5, v0, 0.5, v1, 0, v1) and
// REDUCE2(REDUCE2(v00, v01), REDUCE2(v10, v11)).
enum Preset { kSrgba8 = 1, kRgba32f = 2, kRgba16f = 3, kRgba16Unorm = 4 };

uint32_t texelBytes(int preset) {
  return preset == kSrgba8 ? 4 : preset == kRgba32f ? 16 : (preset == kRgba16f || preset == kRgba16Unorm) ? 8 : 0;
}

// The reductions of the run in progress are the reference's defaults derived
// from REDUCE (kRgba16Unorm) instead of the sRGBA8 preset's own macros.
thread_local bool t_derivedReductions = false;

struct Image {
  int preset;
  uint32_t bpp;
  uint8_t* base;
  std::vector<uint64_t> off;
  std::vector<uint32_t> w, h;
  Image(int p, uint32_t W, uint32_t H, uint32_t levels, uint8_t* b) : preset(p), bpp(texelBytes(p)), base(b) {
    uint64_t o = 0;
    for (uint32_t k = 0; k < levels; ++k) {
      uint32_t lw = std::max(W >> k, 1u), lh = std::max(H >> k, 1u);
      w.push_back(lw);
      h.push_back(lh);
      off.push_back(o);
      o += (uint64_t)lw * lh * bpp;
    }
  }
  uint8_t* at(uint32_t level, uint32_t x, uint32_t y) const {
    return base + off[level] + ((uint64_t)y * w[level] + x) * bpp;
  }
  // NVPRO_PYRAMID_LOAD: texelFetch (preamble.glsl:21-22).
  Vec4 load(uint32_t level, uint32_t x, uint32_t y) const {
    const uint8_t* p = at(level, x, y);
    Vec4 r;
    if (preset == kSrgba8) {
      const SrgbTables& t = tables();
      r.v[0] = t.decode[p[0]];
      r.v[1] = t.decode[p[1]];
      r.v[2] = t.decode[p[2]];
      r.v[3] = t.alpha[p[3]];
    } else if (preset == kRgba32f) {
      std::memcpy(r.v, p, 16);
    } else if (preset == kRgba16Unorm) {
      for (int c = 0; c < 4; ++c) {
        uint16_t u;
        std::memcpy(&u, p + 2 * c, 2);
        r.v[c] = (float)u / 65535.0f;
      }
    } else {
      for (int c = 0; c < 4; ++c) {
        uint16_t hv;
        std::memcpy(&hv, p + 2 * c, 2);
        r.v[c] = halfToFloat(hv);
      }
    }
    return r;
  }
  // NVPRO_PYRAMID_STORE: imageStore(srgbFromLinearVec(v)) (preamble.glsl:27-28,110-128).
  void store(uint32_t level, uint32_t x, uint32_t y, const Vec4& v) const {
    uint8_t* p = at(level, x, y);
    if (preset == kSrgba8) {
      p[0] = (uint8_t)srgbEncode(v.v[0]);
      p[1] = (uint8_t)srgbEncode(v.v[1]);
      p[2] = (uint8_t)srgbEncode(v.v[2]);
      p[3] = (uint8_t)alphaEncode(v.v[3]);
    } else if (preset == kRgba32f) {
      std::memcpy(p, v.v, 16);
    } else if (preset == kRgba16Unorm) {
      for (int c = 0; c < 4; ++c) {
        const float x = std::fmin(std::fmax(v.v[c], 0.0f), 1.0f);
        const float t = x * 65535.0f + 0.5f;  // two roundings (-ffp-contract=off)
        const uint16_t u = (uint16_t)(uint32_t)t;
        std::memcpy(p + 2 * c, &u, 2);
      }
    } else {
      for (int c = 0; c < 4; ++c) {
        uint16_t hv = floatToHalf(v.v[c]);
        std::memcpy(p + 2 * c, &hv, 2);
      }
    }
  }
};

// NVPRO_PYRAMID_REDUCE: a0 * v0 + a1 * v1 + a2 * v2 (preamble.glsl:24-25).
Vec4 reduce3(float a0, const Vec4& v0, float a1, const Vec4& v1, float a2, const Vec4& v2) {
  Vec4 r;
  for (int c = 0; c < 4; ++c) {
    float p0 = a0 * v0.v[c];
    float p1 = a1 * v1.v[c];
    float p2 = a2 * v2.v[c];
    float s = p0 + p1;
    r.v[c] = s + p2;
  }
  return r;
}
// NVPRO_PYRAMID_REDUCE2: 0.5 * (v0 + v1) (preamble.glsl:35).
Vec4 reduce2(const Vec4& v0, const Vec4& v1) {
  if (t_derivedReductions) return reduce3(0.5f, v0, 0.5f, v1, 0.0f, v1);
  Vec4 r;
  for (int c = 0; c < 4; ++c) r.v[c] = 0.5f * (v0.v[c] + v1.v[c]);
  return r;
}
// NVPRO_PYRAMID_REDUCE4: 0.25 * ((v00 + v01) + (v10 + v11)) (preamble.glsl:37-38).
Vec4 reduce4(const Vec4& v00, const Vec4& v01, const Vec4& v10, const Vec4& v11) {
  if (t_derivedReductions) return reduce2(reduce2(v00, v01), reduce2(v10, v11));
  Vec4 r;
  for (int c = 0; c < 4; ++c) {
    float a = v00.v[c] + v01.v[c];
    float b = v10.v[c] + v11.v[c];
    r.v[c] = 0.25f * (a + b);
  }
  return r;
}

// Which pairs the fast pipeline adds first when it builds level L+k of an
// n-level dispatch (k = 1..n).  'V' = vertical pairs first,
// 0.25*((TL+BL)+(TR+BR)); 'H' = horizontal pairs first, 0.25*((TL+TR)+(BL+BR)).
//  k=1: LOAD_REDUCE4 passes (0,0),(0,1),(1,0),(1,1) (nvpro_pyramid.glsl:180-188): V.
//  n=6, k=2: REDUCE4(s00, s01=(0,1), s10=(1,0), s11) (:342): V.
//  shuffle stages xor 1,2,3 / xor 4,8,12, lane bit 0 / bit 2 = x (:349-350,:308-309): H.
//  shared-memory tail, smem[+1] = right, smem[+2] = below (:487-491,:509-513): V;
//  its final shuffle xor 1 = x, xor 2 = y, REDUCE4(in00, in01=y, ...) (:519-526): V.
char fastOrder(uint32_t n, uint32_t k) {
  if (k == 1) return 'V';
  if (n == 6) return (k == 2 || k >= 5) ? 'V' : 'H';
  if (n >= 4) return k >= 4 ? 'V' : 'H';
  return 'H';
}

// Shared-memory formats of the sRGBA8 preset (srgba8_mipmap_preamble.glsl:60-108).
enum SharedFormat { kSharedFp32 = 0, kSharedSrgb = 1, kSharedF16 = 2 };

// The level (relative to L) whose values an n-level dispatch hands on through
// shared memory, 0 if none.  Fast: handleTile_ fills subLevelCount_ = 4 (n = 6)
// or 3 (n = 4, 5) levels and writes the last one to sharedTile_
// (nvpro_pyramid.glsl:440-462, :393-396); the tail reads it back (:487-512).
// General, two levels: level L+1 goes to sharedLevel_ (:717) and level L+2
// reads it back (:664).
uint32_t handoffLevel(bool fast, uint32_t n) {
  if (fast) return n == 6 ? 4 : n >= 4 ? 3 : 0;
  return n == 2 ? 1 : 0;
}

// NVPRO_PYRAMID_SHARED_STORE then NVPRO_PYRAMID_SHARED_LOAD of a value.
// SRGB_SHARED packs the sRGB code (srgbPack, preamble.glsl:91-99) and decodes
// it again (srgbUnpack, :81-88); GLSL leaves pow()'s precision and the
// rounding of halves in packUnorm4x8 to the implementation, so the code here
// is the exact one of the STORE encoding and the decode is the LOAD table.
// F16_SHARED: f16vec4(v), round to nearest even, and back (:103-108).
Vec4 sharedRoundTrip(int fmt, const Vec4& v) {
  if (fmt == kSharedFp32) return v;
  Vec4 r;
  if (fmt == kSharedSrgb) {
    const SrgbTables& t = tables();
    for (int c = 0; c < 3; ++c) r.v[c] = t.decode[srgbEncode(v.v[c])];
    r.v[3] = t.alpha[alphaEncode(v.v[3])];
  } else {
    for (int c = 0; c < 4; ++c) r.v[c] = halfToFloat(floatToHalf(v.v[c]));
  }
  return r;
}

// Fast pipeline dispatch (nvpro_pyramid.glsl:401-532): levels L+1..L+n from
// square tiles of edge 2^n of level L; all values inside the dispatch stay FP32
// except the hand-off level of a pipeline with a shared format (sharedFmt).
void fastDispatch(const Image& img, uint32_t L, uint32_t n, uint64_t groups, int sharedFmt) {
  const uint32_t W = img.w[L], H = img.h[L];
  const uint32_t T = 1u << n;
  const uint64_t tilesX = W >> n, tilesY = H >> n;
  const uint64_t tilesPerGroup = (n > 5 ? 4096u : 1024u) >> (2 * n);
  const uint64_t limit = std::min<uint64_t>(tilesX * tilesY, groups * std::max<uint64_t>(tilesPerGroup, 1));
  std::vector<Vec4> cur, next;
  const uint32_t handoff = sharedFmt != kSharedFp32 ? handoffLevel(true, n) : 0;
  for (uint64_t t = 0; t < limit; ++t) {
    const uint32_t tx = (uint32_t)(t % tilesX), ty = (uint32_t)(t / tilesX);
    uint32_t e = T / 2;  // edge of the level L+1 tile
    cur.assign((size_t)e * e, Vec4{});
    for (uint32_t y = 0; y < e; ++y)
      for (uint32_t x = 0; x < e; ++x) {
        const uint32_t sx = tx * T + 2 * x, sy = ty * T + 2 * y;
        Vec4 v = reduce4(img.load(L, sx, sy), img.load(L, sx, sy + 1), img.load(L, sx + 1, sy),
                         img.load(L, sx + 1, sy + 1));
        cur[(size_t)y * e + x] = v;
        img.store(L + 1, tx * e + x, ty * e + y, v);
      }
    for (uint32_t k = 2; k <= n; ++k) {
      const uint32_t ne = e / 2;
      next.assign((size_t)ne * ne, Vec4{});
      const bool vert = fastOrder(n, k) == 'V';
      for (uint32_t y = 0; y < ne; ++y)
        for (uint32_t x = 0; x < ne; ++x) {
          const Vec4& tl = cur[(size_t)(2 * y) * e + 2 * x];
          const Vec4& tr = cur[(size_t)(2 * y) * e + 2 * x + 1];
          const Vec4& bl = cur[(size_t)(2 * y + 1) * e + 2 * x];
          const Vec4& br = cur[(size_t)(2 * y + 1) * e + 2 * x + 1];
          Vec4 v = vert ? reduce4(tl, bl, tr, br) : reduce4(tl, tr, bl, br);
          next[(size_t)y * ne + x] = k == handoff ? sharedRoundTrip(sharedFmt, v) : v;
          img.store(L + k, tx * ne + x, ty * ne + y, v);
        }
      cur.swap(next);
      e = ne;
    }
  }
}

// kernelSizeFromInputSize_ (nvpro_pyramid.glsl:557-561).
uint32_t kernelSize(uint32_t inputSize) { return inputSize == 1 ? 1u : (2u | (inputSize & 1u)); }

struct Weights {
  float w0, w1, w2;
};
// nvpro_pyramid.glsl:582-586 and :639-643.
Weights weights(uint32_t dstSize, uint32_t dstCoord) {
  const float n = (float)dstSize;
  const float denom = 2.0f * n + 1.0f;
  const float rcp = 1.0f / denom;
  Weights w;
  w.w0 = rcp * (n - (float)dstCoord);
  w.w1 = rcp * n;
  w.w2 = (1.0f - w.w0) - w.w1;
  return w;
}

// reduceStoreSample_ (nvpro_pyramid.glsl:575-656) without the store, with a
// loader returning the FP32 sample at offsets (dx, dy) from the source corner.
template <typename Loader>
Vec4 reduceSample(Loader&& ld, uint32_t kx, uint32_t ky, uint32_t dstW, uint32_t dstH, uint32_t x,
                  uint32_t y) {
  const Weights wy = weights(dstH, y);
  Vec4 h[3];
  for (uint32_t c = 0; c < kx; ++c) {
    if (ky == 3)
      h[c] = reduce3(wy.w0, ld(c, 0), wy.w1, ld(c, 1), wy.w2, ld(c, 2));
    else if (ky == 2)
      h[c] = reduce2(ld(c, 0), ld(c, 1));
    else
      h[c] = ld(c, 0);
  }
  if (kx == 3) {
    const Weights wx = weights(dstW, x);
    return reduce3(wx.w0, h[0], wx.w1, h[1], wx.w2, h[2]);
  }
  if (kx == 2) return reduce2(h[0], h[1]);
  return h[0];
}

// General pipeline dispatch (nvpro_pyramid.glsl:824-882), 1 or 2 levels.
void generalDispatch(const Image& img, uint32_t L, uint32_t n, uint64_t groups, int sharedFmt) {
  const uint32_t sw = img.w[L], sh = img.h[L];
  const uint32_t w1 = img.w[L + 1], h1 = img.h[L + 1];
  const uint32_t kx = kernelSize(sw), ky = kernelSize(sh);
  auto levelSample = [&](uint32_t x, uint32_t y) {
    return reduceSample([&](uint32_t dx, uint32_t dy) { return img.load(L, 2 * x + dx, 2 * y + dy); }, kx,
                        ky, w1, h1, x, y);
  };
  if (n == 1) {
    const uint64_t total = (uint64_t)w1 * h1;
    const uint64_t limit = std::min<uint64_t>(total, groups * 128u);
    for (uint64_t i = 0; i < limit; ++i) {
      const uint32_t x = (uint32_t)(i % w1), y = (uint32_t)(i / w1);
      img.store(L + 1, x, y, levelSample(x, y));
    }
    return;
  }
  // Two levels: 8x8 tiles of level L+2, each built from a 16..17 square
  // window of level L+1 kept in FP32 (fillIntermediateTile_, :732-781).
  const uint32_t w2 = img.w[L + 2], h2 = img.h[L + 2];
  const uint32_t fkx = kernelSize(w1), fky = kernelSize(h1);
  const uint32_t winW = fkx == 3 ? 17 : 16, winH = fky == 3 ? 17 : 16;
  const uint64_t tilesX = (w2 + 7) / 8, tilesY = (h2 + 7) / 8;
  const uint64_t limit = std::min<uint64_t>(tilesX * tilesY, groups);
  std::vector<Vec4> lvl1((size_t)w1 * h1);
  std::vector<uint8_t> have((size_t)w1 * h1, 0);
  for (uint64_t t = 0; t < limit; ++t) {
    const uint32_t tx = (uint32_t)(t % tilesX), ty = (uint32_t)(t / tilesX);
    for (uint32_t j = 0; j < winH; ++j)
      for (uint32_t i = 0; i < winW; ++i) {
        const uint32_t x = tx * 16 + i, y = ty * 16 + j;
        if (x >= w1 || y >= h1) continue;
        const size_t idx = (size_t)y * w1 + x;
        if (!have[idx]) {
          const Vec4 v = levelSample(x, y);
          lvl1[idx] = sharedRoundTrip(sharedFmt, v);
          have[idx] = 1;
          img.store(L + 1, x, y, v);
        }
      }
    for (uint32_t j = 0; j < 8; ++j)
      for (uint32_t i = 0; i < 8; ++i) {
        const uint32_t x = tx * 8 + i, y = ty * 8 + j;
        if (x >= w2 || y >= h2) continue;
        Vec4 v = reduceSample([&](uint32_t dx, uint32_t dy) { return lvl1[(size_t)(2 * y + dy) * w1 + 2 * x + dx]; },
                              fkx, fky, w2, h2, x, y);
        img.store(L + 2, x, y, v);
      }
  }
}

// Linear blit of level L to L + 1 (vkCmdBlitImage, VK_FILTER_LINEAR; the
// fallback of demo_app/mipmap_pipelines.cpp:408-423), with the library's
// pinned FP32 filter: per axis scale = src / dst, u = (x + 0.5) * scale - 0.5,
// i = floor(u), a = u - i, taps i and i + 1 clamped to the edge; rows lerped
// first (t0 * (1 - a) + t1 * a), then the column; STORE encoding.
void blitLevel(const Image& img, uint32_t L) {
  const uint32_t sw = img.w[L], sh = img.h[L], dw = img.w[L + 1], dh = img.h[L + 1];
  struct Tap {
    uint32_t i0, i1;
    float a;
  };
  auto axis = [](uint32_t x, uint32_t src, uint32_t dst) {
    const float scale = (float)src / (float)dst;
    const float t = (float)x + 0.5f;
    const float u = t * scale - 0.5f;
    const float f = std::floor(u);
    Tap r;
    r.a = u - f;
    const int i = (int)f;
    r.i0 = (uint32_t)std::min(std::max(i, 0), (int)src - 1);
    r.i1 = (uint32_t)std::min(std::max(i + 1, 0), (int)src - 1);
    return r;
  };
  auto lerp = [](const Vec4& t0, const Vec4& t1, float a) {
    const float b = 1.0f - a;
    Vec4 r;
    for (int c = 0; c < 4; ++c) {
      const float p0 = t0.v[c] * b;
      const float p1 = t1.v[c] * a;
      r.v[c] = p0 + p1;
    }
    return r;
  };
  for (uint32_t y = 0; y < dh; ++y)
    for (uint32_t x = 0; x < dw; ++x) {
      const Tap ax = axis(x, sw, dw), ay = axis(y, sh, dh);
      const Vec4 r0 = lerp(img.load(L, ax.i0, ay.i0), img.load(L, ax.i1, ay.i0), ax.a);
      const Vec4 r1 = lerp(img.load(L, ax.i0, ay.i1), img.load(L, ax.i1, ay.i1), ax.a);
      img.store(L + 1, x, y, lerp(r0, r1, ay.a));
    }
}

uint32_t fullLevels(uint32_t w, uint32_t h) {
  uint32_t m = 0;
  while (w != 0 || h != 0) {
    w >>= 1;
    h >>= 1;
    ++m;
  }
  return m;
}

// ---- the reference CPU generator, restated (include/mipmap_storage.hpp) ----

// shaders/srgb.h:18-28 (FP32 arithmetic, powf).
float refLinearFromSrgb(uint32_t arg) {
  arg = arg > 255u ? 255u : arg;
  float u = (float)arg * (1.0F / 255.0F);
  if (u <= 0.04045F) return u * (25.0F / 323.0F);
  float t = 200.0F * u;
  t = t + 11.0F;
  t = t * (1.0F / 211.0F);
  return powf(t, 2.4F);
}
// shaders/srgb.h:30-41.
uint32_t refSrgbFromLinear(float arg) {
  float srgb;
  if (arg <= 0.0031308F) {
    srgb = (323.0F / 25.0F) * arg;
  } else {
    float p = powf(arg, 1.0F / 2.4F);
    srgb = 1.055F * p;
    srgb = srgb - 0.055F;
  }
  float s = srgb * 255.0F;
  s = s + 0.5F;
  s = std::min(std::max(s, 0.0F), 255.0F);
  return (uint32_t)s;
}

// MipmapStorage::generateLevel (include/mipmap_storage.hpp:246-392) for the
// sRGBA8 converters of cpuGenerateMipmaps_sRGBA (:395-414).
void refcpuLevel(const Image& img, uint32_t level) {
  const uint32_t sw = img.w[level - 1], sh = img.h[level - 1];
  const uint32_t dw = img.w[level], dh = img.h[level];
  const bool wEven = !(sw & 1), hEven = !(sh & 1);
  auto toLinear = [&](uint32_t x, uint32_t y) {
    const uint8_t* p = img.at(level - 1, x, y);
    Vec4 r;
    r.v[0] = refLinearFromSrgb(p[0]);
    r.v[1] = refLinearFromSrgb(p[1]);
    r.v[2] = refLinearFromSrgb(p[2]);
    r.v[3] = (float)p[3] * (1.F / 255.F);
    return r;
  };
  auto mac = [](Vec4& acc, const Vec4& s, float wt) {
    for (int c = 0; c < 4; ++c) {
      float p = s.v[c] * wt;
      acc.v[c] = acc.v[c] + p;
    }
  };
  for (uint32_t y = 0; y < dh; ++y)
    for (uint32_t x = 0; x < dw; ++x) {
      // Rows/columns that the reference reads: 2 for even sizes, 3 for odd
      // sizes, 1 for a size of 1.
      const bool has1x = wEven || sw != 1, has1y = hEven || sh != 1;
      const bool has2x = !wEven && sw != 1, has2y = !hEven && sh != 1;
      Vec4 s[3][3] = {};  // s[col][row]
      s[0][0] = toLinear(2 * x, 2 * y);
      if (has1x) s[1][0] = toLinear(2 * x + 1, 2 * y);
      if (has1y) {
        s[0][1] = toLinear(2 * x, 2 * y + 1);
        if (has1x) s[1][1] = toLinear(2 * x + 1, 2 * y + 1);
      }
      if (has2x) {
        s[2][0] = toLinear(2 * x + 2, 2 * y);
        // The reference also reads (2, 1) when the height is 1; that value
        // is never used, so it is skipped here (it would lie outside the level).
        if (has1y) s[2][1] = toLinear(2 * x + 2, 2 * y + 1);
        if (has2y) s[2][2] = toLinear(2 * x + 2, 2 * y + 2);
      }
      if (has2y) {
        s[0][2] = toLinear(2 * x, 2 * y + 2);
        s[1][2] = toLinear(2 * x + 1, 2 * y + 2);
      }
      Vec4 col[3] = {};
      if (hEven) {
        mac(col[0], s[0][0], 0.5F);
        mac(col[0], s[0][1], 0.5F);
        mac(col[1], s[1][0], 0.5F);
        mac(col[1], s[1][1], 0.5F);
        if (!wEven) {
          mac(col[2], s[2][0], 0.5F);
          mac(col[2], s[2][1], 0.5F);
        }
      } else if (sh == 1) {
        col[0] = s[0][0];
        if (has1x) col[1] = s[1][0];
        if (!wEven) col[2] = s[2][0];
      } else {
        const float n = (float)dh;
        const float rcp = 1.0F / (2 * n + 1);
        const float w0 = rcp * (n - (float)y), w1 = rcp * n, w2 = rcp * (float)(1 + y);
        for (int c = 0; c < 3; ++c) {
          if (c == 1 && !has1x) continue;
          if (c == 2 && wEven) continue;
          mac(col[c], s[c][0], w0);
          mac(col[c], s[c][1], w1);
          mac(col[c], s[c][2], w2);
        }
      }
      Vec4 out = {};
      if (wEven) {
        mac(out, col[0], 0.5F);
        mac(out, col[1], 0.5F);
      } else if (sw == 1) {
        out = col[0];
      } else {
        const float n = (float)dw;
        const float rcp = 1.0F / (2 * n + 1);
        const float w0 = rcp * (n - (float)x), w1 = rcp * n, w2 = rcp * (float)(1 + x);
        mac(out, col[0], w0);
        mac(out, col[1], w1);
        mac(out, col[2], w2);
      }
      uint8_t* p = img.at(level, x, y);
      float a = out.v[3] * 255.F;
      a = std::min(std::max(a, 0.F), 255.F);
      p[0] = (uint8_t)refSrgbFromLinear(out.v[0]);
      p[1] = (uint8_t)refSrgbFromLinear(out.v[1]);
      p[2] = (uint8_t)refSrgbFromLinear(out.v[2]);
      p[3] = (uint8_t)a;
    }
}

// FP64 version of the per-level operator (exact weights), for float presets.
void f64Level(double* base, const std::vector<uint64_t>& off, const std::vector<uint32_t>& w,
              const std::vector<uint32_t>& h, uint32_t level) {
  const uint32_t sw = w[level - 1], sh = h[level - 1], dw = w[level], dh = h[level];
  const uint32_t kx = kernelSize(sw), ky = kernelSize(sh);
  const double* src = base + off[level - 1] * 4;
  double* dst = base + off[level] * 4;
  auto wts = [](uint32_t k, uint32_t n, uint32_t i, double* o) {
    if (k == 1) {
      o[0] = 1;
    } else if (k == 2) {
      o[0] = o[1] = 0.5;
    } else {
      const double d = 2.0 * n + 1.0;
      o[0] = (n - (double)i) / d;
      o[1] = n / d;
      o[2] = (1.0 + i) / d;
    }
  };
  for (uint32_t y = 0; y < dh; ++y)
    for (uint32_t x = 0; x < dw; ++x) {
      double wx[3], wy[3];
      wts(kx, dw, x, wx);
      wts(ky, dh, y, wy);
      for (int c = 0; c < 4; ++c) {
        double acc = 0;
        for (uint32_t j = 0; j < ky; ++j)
          for (uint32_t i = 0; i < kx; ++i)
            acc += wx[i] * wy[j] * src[((uint64_t)(2 * y + j) * sw + 2 * x + i) * 4 + c];
        dst[((uint64_t)y * dw + x) * 4 + c] = acc;
      }
    }
}

}  // namespace

extern "C" {

uint32_t orc_full_level_count(uint32_t w, uint32_t h) { return fullLevels(w, h); }

// Packed level offsets in bytes; writes levels + 1 values.
int orc_packed_offsets(uint32_t w, uint32_t h, uint32_t levels, uint32_t bpp, uint64_t* out) {
  uint64_t o = 0;
  for (uint32_t k = 0; k < levels; ++k) {
    out[k] = o;
    o += (uint64_t)std::max(w >> k, 1u) * std::max(h >> k, 1u) * bpp;
  }
  out[levels] = o;
  return 0;
}

// The default dispatch schedule (nvpro_pyramid_dispatch.hpp:109-304).
// fastDiv/fastMax: template arguments of the fast dispatcher (4, 6 by default);
// hasFast = 0 means pipelines.fastPipeline == VK_NULL_HANDLE.
// Writes isFast, push constant and workgroup count per dispatch; returns the
// number of dispatches or -1 if maxRecords is too small.
int orc_default_schedule(uint32_t w, uint32_t h, uint32_t mipLevels, int hasFast, uint32_t fastDiv,
                         uint32_t fastMax, uint32_t* isFast, uint32_t* pc, uint32_t* groups, int maxRecords) {
  if (mipLevels == 0) mipLevels = fullLevels(w, h);
  uint32_t level = 0, remaining = mipLevels - 1, x = w, y = h;
  int n = 0;
  while (remaining != 0) {
    if (n >= maxRecords) return -1;
    uint32_t done = 0;
    if (hasFast && x % fastDiv == 0 && y % fastDiv == 0) {
      uint32_t tx = x, ty = y;
      while (tx % 2 == 0 && ty % 2 == 0 && done < remaining && done < fastMax) {
        tx /= 2;
        ty /= 2;
        ++done;
      }
      const uint32_t shift = done > 5 ? 12 : 10, mask = done > 5 ? 4095 : 1023;
      isFast[n] = 1;
      pc[n] = level << 5 | done;
      groups[n] = (x * y + mask) >> shift;  // 32-bit, as the reference computes it
    }
    if (done == 0) {
      done = remaining >= 2 ? 2 : remaining;
      const uint32_t dw = std::max(x >> done, 1u), dh = std::max(y >> done, 1u);
      isFast[n] = 0;
      pc[n] = level << 5 | done;
      groups[n] = done == 1 ? (dw * dh + 127) / 128 : ((dw + 7) / 8) * ((dh + 7) / 8);
    }
    ++n;
    level += done;
    remaining -= done;
    x = std::max(x >> done, 1u);
    y = std::max(y >> done, 1u);
  }
  return n;
}

// Run a dispatch sequence (shader semantics) on a packed image whose level 0
// is filled.  preset: 1 sRGBA8, 2 RGBA32F, 3 RGBA16F, 4 RGBA 16-bit unorm
// (the tests' custom functor set).  isFast: 1 fast
// dispatch, 0 general dispatch, 2 linear blit of one level.  fastShared /
// generalShared: shared-memory format of the fast / general pipeline
// (0 FP32, 1 SRGB_SHARED, 2 F16_SHARED; sRGBA8 only).
int orc_run_ex(int preset, int fastShared, int generalShared, uint32_t w, uint32_t h, uint32_t mipLevels,
               const uint32_t* isFast, const uint32_t* pc, const uint32_t* groups, int count, uint8_t* packed) {
  if (texelBytes(preset) == 0 || w == 0 || h == 0) return -1;
  if (fastShared < 0 || fastShared > 2 || generalShared < 0 || generalShared > 2) return -4;
  if ((fastShared || generalShared) && preset != kSrgba8) return -4;
  if (mipLevels == 0) mipLevels = fullLevels(w, h);
  Image img(preset, w, h, mipLevels, packed);
  t_derivedReductions = preset == kRgba16Unorm;
  struct Reset {
    ~Reset() { t_derivedReductions = false; }
  } reset;
  for (int i = 0; i < count; ++i) {
    const uint32_t L = pc[i] >> 5, n = pc[i] & 31u;
    if (n == 0 || L + n >= mipLevels) return -2;
    if (isFast[i] == 2) {  // a linear blit of one level
      if (n != 1) return -3;
      blitLevel(img, L);
    } else if (isFast[i]) {
      if (n > 6 || (img.w[L] % (1u << n)) || (img.h[L] % (1u << n))) return -3;
      fastDispatch(img, L, n, groups[i], fastShared);
    } else {
      if (n > 2) return -3;
      generalDispatch(img, L, n, groups[i], generalShared);
    }
  }
  return 0;
}

int orc_run(int preset, uint32_t w, uint32_t h, uint32_t mipLevels, const uint32_t* isFast, const uint32_t* pc,
            const uint32_t* groups, int count, uint8_t* packed) {
  return orc_run_ex(preset, 0, 0, w, h, mipLevels, isFast, pc, groups, count, packed);
}

// The reference CPU generator (cpuGenerateMipmaps_sRGBA), restated.
int orc_refcpu_srgba8(uint32_t w, uint32_t h, uint8_t* packed) {
  if (w == 0 || h == 0) return -1;
  const uint32_t levels = fullLevels(w, h);
  Image img(kSrgba8, w, h, levels, packed);
  for (uint32_t k = 1; k < levels; ++k) refcpuLevel(img, k);
  return 0;
}

// FP64 pyramid of a packed RGBA double image (level 0 filled).
int orc_f64_pyramid(uint32_t w, uint32_t h, uint32_t mipLevels, double* packed) {
  if (mipLevels == 0) mipLevels = fullLevels(w, h);
  std::vector<uint64_t> off;
  std::vector<uint32_t> lw, lh;
  uint64_t o = 0;
  for (uint32_t k = 0; k < mipLevels; ++k) {
    lw.push_back(std::max(w >> k, 1u));
    lh.push_back(std::max(h >> k, 1u));
    off.push_back(o);
    o += (uint64_t)lw.back() * lh.back();
  }
  for (uint32_t k = 1; k < mipLevels; ++k) f64Level(packed, off, lw, lh, k);
  return 0;
}

void orc_srgb_tables(float* decode, float* alpha, float* thr) {
  const SrgbTables& t = tables();
  std::memcpy(decode, t.decode, sizeof t.decode);
  std::memcpy(alpha, t.alpha, sizeof t.alpha);
  std::memcpy(thr, t.thr, sizeof t.thr);
}

uint32_t orc_srgb_encode(float x) { return srgbEncode(x); }
uint32_t orc_alpha_encode(float a) { return alphaEncode(a); }
float orc_half_to_float(uint16_t h) { return halfToFloat(h); }
uint16_t orc_float_to_half(float f) { return floatToHalf(f); }
float orc_ref_linear_from_srgb(uint32_t c) { return refLinearFromSrgb(c); }
uint32_t orc_ref_srgb_from_linear(float x) { return refSrgbFromLinear(x); }

// Premultiplied-alpha staging (include/scoped_image.hpp:233-255) of n sRGBA8
// texels: a = A * (1.F / 255.F); colour c -> srgbFromLinear(linearFromSrgb(c)
// * a); alpha unchanged.  referenceMath = 1: the reference's FP32 pow()
// formulas (shaders/srgb.h, restated above); 0: the library's pinned exact
// codec (decode table, threshold-count encode).
void orc_premultiply_srgba8(const uint8_t* src, uint8_t* dst, uint64_t n, int referenceMath) {
  const SrgbTables& t = tables();
  for (uint64_t i = 0; i < n; ++i) {
    const uint8_t* s = src + 4 * i;
    uint8_t* d = dst + 4 * i;
    const float alpha = (float)s[3] * (1.F / 255.F);
    uint8_t out[4];
    for (int c = 0; c < 3; ++c) {
      const float lin = referenceMath ? refLinearFromSrgb(s[c]) : t.decode[s[c]];
      const float v = lin * alpha;
      out[c] = (uint8_t)(referenceMath ? refSrgbFromLinear(v) : srgbEncode(v));
    }
    out[3] = s[3];
    std::memcpy(d, out, 4);
  }
}

// Encode an array of floats (for exhaustive comparisons).
void orc_srgb_encode_array(const float* x, uint8_t* out, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) out[i] = (uint8_t)srgbEncode(x[i]);
}

}  // extern "C"
