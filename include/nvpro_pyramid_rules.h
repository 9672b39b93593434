/*
 * nvpro_pyramid_rules.h -- the pure rules of the nvpro_pyramid schedule that
 * every kernel family shares, usable from host and device code (C++ only).
 * Included by nvpro_pyramid_cuda.hpp and by the library's own sources.
 */
#ifndef NVPRO_PYRAMID_RULES_H_
#define NVPRO_PYRAMID_RULES_H_

#include <stdint.h>

#if defined(__CUDACC__)
#define NVPRO_PYRAMID_HD __host__ __device__ __forceinline__
#else
#define NVPRO_PYRAMID_HD inline
#endif

namespace nvpro_pyramid {

/* kernelSizeFromInputSize_ (nvpro_pyramid.glsl:557-561): taps of the general
 * pipeline along an axis whose input level has `inputSize` texels. */
NVPRO_PYRAMID_HD uint32_t kernelSize(uint32_t inputSize) { return inputSize == 1 ? 1u : (2u | (inputSize & 1u)); }

/* Reduction order of the fast pipeline for level L+k of an n-level dispatch:
 * true = vertical pairs first, REDUCE4(TL, BL, TR, BR); false = horizontal
 * pairs first, REDUCE4(TL, TR, BL, BR).  Derived from which operand each
 * REDUCE4 call of nvpro_pyramid.glsl receives: the LOAD_REDUCE4 of level 1
 * (:180-188) and the 2x2 step of 6-level dispatches (:342) pair vertically;
 * the subgroup-shuffle stages (:364-397) pair horizontally; the shared-memory
 * tail (:472-531) pairs vertically. */
NVPRO_PYRAMID_HD bool fastVerticalFirst(uint32_t n, uint32_t k) {
  if (k == 1) return true;
  if (n == 6) return k == 2 || k >= 5;
  if (n >= 4) return k >= 4;
  return false;
}

/* The level (relative to the input level) whose values a dispatch of n levels
 * hands on through the reference's shared memory, or 0 if none: L+3 for fast
 * dispatches of 4 or 5 levels, L+4 for 6 levels (nvpro_pyramid.glsl:440-462),
 * L+1 for two-level general dispatches (:717).  A pipeline's shared format
 * (NVPRO_PYRAMID_SHARED_TYPE / LOAD / STORE) applies to the values of that
 * level, which is itself stored from the unconverted values. */
NVPRO_PYRAMID_HD uint32_t sharedHandoffLevel(bool isFast, uint32_t n) {
  if (isFast) return n == 6 ? 4u : n >= 4 ? 3u : 0u;
  return n == 2 ? 1u : 0u;
}

/* Workgroups of the reference's fast dispatcher that cover every 2^n tile of
 * an n-level fast dispatch over a w x h level (nvpro_pyramid_dispatch.hpp:
 * 234-238: 4096 input samples per group for 6 levels, else 1024). */
NVPRO_PYRAMID_HD uint64_t fastGroupsNeeded(uint32_t w, uint32_t h, uint32_t n) {
  const uint64_t tiles = uint64_t(w >> n) * (h >> n);
  const uint64_t perGroup = (n > 5 ? 4096u : 1024u) >> (2 * n);
  const uint64_t per = perGroup ? perGroup : 1;
  return (tiles + per - 1) / per;
}

}  // namespace nvpro_pyramid

#endif /* NVPRO_PYRAMID_RULES_H_ */
