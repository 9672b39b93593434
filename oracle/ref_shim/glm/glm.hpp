// Minimal stand-in for the parts of glm that the reference's CPU mipmap
// generator (include/mipmap_storage.hpp, shaders/srgb.h) uses: uvec2, uvec3,
// clamp.  TEST INFRASTRUCTURE ONLY (oracle/_ref build).
#pragma once
#include <stdint.h>

namespace glm {
struct uvec2 {
  uint32_t x = 0, y = 0;
  uvec2() = default;
  uvec2(uint32_t x_, uint32_t y_) : x(x_), y(y_) {}
  bool operator==(const uvec2& o) const { return x == o.x && y == o.y; }
};
struct uvec3 {
  uint32_t x = 0, y = 0, z = 0;
  uvec3() = default;
  uvec3(uint32_t x_, uint32_t y_, uint32_t z_) : x(x_), y(y_), z(z_) {}
};
template <typename T>
T clamp(T v, T lo, T hi) {
  T m = v < lo ? lo : v;  // max(v, lo)
  return hi < m ? hi : m; // min(., hi)
}
}  // namespace glm
