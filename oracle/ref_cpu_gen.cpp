// ref_cpu_gen.cpp -- TEST INFRASTRUCTURE ONLY.
// C entry points around the reference's own CPU mipmap generator
// (include/mipmap_storage.hpp:395-414, shaders/srgb.h), compiled from the
// reference sources into oracle/_ref/libref_cpu.so by oracle/Makefile.
// Used to pin oracle/pyr_oracle.cpp and to make tests/golden fixtures.
#include <cstring>

#include "include/mipmap_storage.hpp"

extern "C" {

// Full chain of a w x h sRGBA8 image.  `packed` holds level 0 on entry and all
// levels (MipmapStorage layout) on return.  Returns the level count.
int ref_cpu_generate_srgba8(uint32_t w, uint32_t h, uint8_t* packed) {
  MipmapStorage<uint8_t, 4> mips(w, h);
  std::memcpy(mips.levelData(0), packed, mips.getLevelByteSize(0));
  cpuGenerateMipmaps_sRGBA(&mips);
  const auto& offsets = mips.getLevelOffsets();
  for (uint32_t k = 0; k < offsets.size(); ++k)
    std::memcpy(packed + offsets[k] * 4, mips.levelData(k), mips.getLevelByteSize(k));
  return (int)offsets.size();
}

// Worst per-channel delta between two packed pyramids over levels >= 1
// (MipmapStorage::compare, include/mipmap_storage.hpp:146-202).
int ref_cpu_compare(uint32_t w, uint32_t h, const uint8_t* a, const uint8_t* b, uint32_t* outXYLC) {
  MipmapStorage<uint8_t, 4> mips(w, h);
  const auto& offsets = mips.getLevelOffsets();
  for (uint32_t k = 0; k < offsets.size(); ++k)
    std::memcpy(mips.levelData(k), a + offsets[k] * 4, mips.getLevelByteSize(k));
  glm::uvec3 coord;
  uint32_t channel = 0;
  int delta = mips.compare(b, &coord, &channel);
  if (outXYLC) {
    outXYLC[0] = coord.x;
    outXYLC[1] = coord.y;
    outXYLC[2] = coord.z;
    outXYLC[3] = channel;
  }
  return delta;
}

float ref_linear_from_srgb(uint32_t c) { return linearFromSrgb(c); }
uint32_t ref_srgb_from_linear(float x) { return srgbFromLinear(x); }
}
