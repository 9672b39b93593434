// host_io.cpp -- debugging I/O of sRGBA8 levels in host memory: TGA files.
//
// The reference writes every level of a pyramid held in its packed
// MipmapStorage layout to TGA files (writeMipmapsTga,
// include/mipmap_storage.hpp:436-479): level 0 to the given name and level k
// to the name with ".k" before the extension, the big levels on threads.
// nvproPyramidWriteLevelsTga does the same for a packed chain in host memory
// (the caller copies it from the device).  The files are uncompressed 32-bit
// TGA (image type 2, top-left origin, 8 alpha bits).  nvproPyramidReadTga
// reads 24- and 32-bit true-colour TGA, uncompressed or run-length encoded,
// either origin, into top-left RGBA8 rows -- enough to load a base level
// without an image library.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/nvpro_pyramid_cuda.h"
#include "internal.h"

using namespace nvpyr;

namespace {

NvproPyramidResult ioFail(NvproPyramidResult r, const std::string& what) {
  setLastError(what.c_str());
  return r;
}

struct File {
  FILE* f;
  explicit File(FILE* p) : f(p) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

NvproPyramidResult writeOne(const char* path, const uint8_t* rgba, uint32_t w, uint32_t h, uint64_t pitch) {
  if (w == 0 || h == 0 || w > 0xFFFF || h > 0xFFFF)
    return ioFail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "TGA sides are 1..65535 (got " + std::to_string(w) + "x" +
                                                            std::to_string(h) + ")");
  File file(std::fopen(path, "wb"));
  if (!file.f) return ioFail(NVPRO_PYRAMID_ERROR_IO, std::string("cannot open ") + path + " for writing");
  uint8_t hdr[18] = {};
  hdr[2] = 2;  // uncompressed true-colour
  hdr[12] = uint8_t(w);
  hdr[13] = uint8_t(w >> 8);
  hdr[14] = uint8_t(h);
  hdr[15] = uint8_t(h >> 8);
  hdr[16] = 32;
  hdr[17] = 0x28;  // top-left origin, 8 attribute (alpha) bits
  bool ok = std::fwrite(hdr, 1, sizeof hdr, file.f) == sizeof hdr;
  std::vector<uint8_t> row(size_t(w) * 4);
  for (uint32_t y = 0; ok && y < h; ++y) {
    const uint8_t* src = rgba + y * pitch;
    for (uint32_t x = 0; x < w; ++x) {  // RGBA -> BGRA
      row[4 * x + 0] = src[4 * x + 2];
      row[4 * x + 1] = src[4 * x + 1];
      row[4 * x + 2] = src[4 * x + 0];
      row[4 * x + 3] = src[4 * x + 3];
    }
    ok = std::fwrite(row.data(), 1, row.size(), file.f) == row.size();
  }
  if (!ok) return ioFail(NVPRO_PYRAMID_ERROR_IO, std::string("write failed: ") + path);
  return NVPRO_PYRAMID_SUCCESS;
}

uint32_t levelDim(uint32_t base, uint32_t k) {
  const uint32_t d = k >= 32 ? 0u : base >> k;
  return d ? d : 1u;
}

}  // namespace

extern "C" {

NvproPyramidResult nvproPyramidWriteTga(const char* path, const void* rgba8, uint32_t width, uint32_t height,
                                        uint64_t rowPitchBytes) {
  if (!path || !rgba8) return ioFail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "null path or pixels");
  const uint64_t pitch = rowPitchBytes ? rowPitchBytes : uint64_t(width) * 4;
  if (pitch < uint64_t(width) * 4) return ioFail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "row pitch below 4 * width");
  return writeOne(path, static_cast<const uint8_t*>(rgba8), width, height, pitch);
}

NvproPyramidResult nvproPyramidWriteLevelsTga(const char* baseFilename, const void* packed, uint32_t width,
                                              uint32_t height, uint32_t levelCount) {
  if (!baseFilename || !packed) return ioFail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "null file name or levels");
  const uint32_t full = nvproPyramidFullLevelCount(width, height);
  if (levelCount == 0) levelCount = full;
  if (width == 0 || height == 0 || levelCount > full)
    return ioFail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "bad size or level count");
  // the extension is the last dot of the file name (the reference looks for
  // the last dot of the whole path, which may be a directory's)
  const char* slash = std::strrchr(baseFilename, '/');
  const char* dot = std::strrchr(slash ? slash : baseFilename, '.');
  const std::string prefix = dot ? std::string(baseFilename, dot - baseFilename + 1) : std::string(baseFilename);
  const std::string suffix = dot ? std::string(dot) : std::string();
  std::vector<uint64_t> off(levelCount + 1);
  if (nvproPyramidPackedLayout(width, height, levelCount, 4, off.data()) != NVPRO_PYRAMID_SUCCESS)
    return NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT;
  std::vector<NvproPyramidResult> results(levelCount, NVPRO_PYRAMID_SUCCESS);
  std::vector<std::string> errors(levelCount);
  auto writeLevel = [&](uint32_t k) {
    const std::string name = k == 0 ? std::string(baseFilename) : prefix + std::to_string(k) + suffix;
    const uint32_t w = levelDim(width, k), h = levelDim(height, k);
    results[k] = writeOne(name.c_str(), static_cast<const uint8_t*>(packed) + off[k], w, h, uint64_t(w) * 4);
    if (results[k] != NVPRO_PYRAMID_SUCCESS) errors[k] = nvproPyramidLastError();
  };
  // the levels above the 8 smallest on threads, as the reference does
  const uint32_t parallel = levelCount > 8 ? levelCount - 8 : 0;
  std::vector<std::thread> threads;
  for (uint32_t k = 0; k < parallel; ++k) threads.emplace_back(writeLevel, k);
  for (uint32_t k = parallel; k < levelCount; ++k) writeLevel(k);
  for (std::thread& t : threads) t.join();
  for (uint32_t k = 0; k < levelCount; ++k)
    if (results[k] != NVPRO_PYRAMID_SUCCESS) return ioFail(results[k], errors[k]);
  return NVPRO_PYRAMID_SUCCESS;
}

NvproPyramidResult nvproPyramidReadTga(const char* path, void* rgba8, uint64_t capacityBytes, uint32_t* pWidth,
                                       uint32_t* pHeight) {
  if (!path || !pWidth || !pHeight) return ioFail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "null argument");
  File file(std::fopen(path, "rb"));
  if (!file.f) return ioFail(NVPRO_PYRAMID_ERROR_IO, std::string("cannot open ") + path);
  uint8_t hdr[18];
  if (std::fread(hdr, 1, 18, file.f) != 18) return ioFail(NVPRO_PYRAMID_ERROR_IO, "truncated TGA header");
  const uint32_t idLen = hdr[0], mapType = hdr[1], type = hdr[2], bpp = hdr[16], desc = hdr[17];
  const uint32_t w = hdr[12] | uint32_t(hdr[13]) << 8, h = hdr[14] | uint32_t(hdr[15]) << 8;
  if (mapType != 0 || (type != 2 && type != 10) || (bpp != 24 && bpp != 32) || (desc & 0x10))
    return ioFail(NVPRO_PYRAMID_ERROR_UNSUPPORTED, "only 24/32-bit true-colour TGA (types 2, 10) is read");
  *pWidth = w;
  *pHeight = h;
  const uint64_t need = uint64_t(w) * h * 4;
  if (!rgba8) return NVPRO_PYRAMID_SUCCESS;  // size query
  if (capacityBytes < need) return ioFail(NVPRO_PYRAMID_ERROR_INVALID_ARGUMENT, "output buffer too small");
  if (std::fseek(file.f, long(idLen), SEEK_CUR) != 0) return ioFail(NVPRO_PYRAMID_ERROR_IO, "truncated TGA");
  const uint32_t px = bpp / 8;
  const uint64_t count = uint64_t(w) * h;
  std::vector<uint8_t> raw(count * px);
  if (type == 2) {
    if (std::fread(raw.data(), 1, raw.size(), file.f) != raw.size())
      return ioFail(NVPRO_PYRAMID_ERROR_IO, "truncated TGA pixel data");
  } else {  // run-length packets: 1 header byte, then one pixel (run) or n pixels (raw)
    uint64_t i = 0;
    while (i < count) {
      const int c = std::fgetc(file.f);
      if (c == EOF) return ioFail(NVPRO_PYRAMID_ERROR_IO, "truncated TGA run");
      const uint64_t n = std::min<uint64_t>((uint64_t(c) & 0x7F) + 1, count - i);
      if (c & 0x80) {
        uint8_t p[4];
        if (std::fread(p, 1, px, file.f) != px) return ioFail(NVPRO_PYRAMID_ERROR_IO, "truncated TGA run");
        for (uint64_t j = 0; j < n; ++j) std::memcpy(&raw[(i + j) * px], p, px);
      } else if (std::fread(&raw[i * px], 1, n * px, file.f) != n * px) {
        return ioFail(NVPRO_PYRAMID_ERROR_IO, "truncated TGA packet");
      }
      i += n;
    }
  }
  const bool topDown = (desc & 0x20) != 0;
  uint8_t* out = static_cast<uint8_t*>(rgba8);
  for (uint32_t y = 0; y < h; ++y) {
    const uint8_t* src = &raw[uint64_t(topDown ? y : h - 1 - y) * w * px];
    uint8_t* dst = out + uint64_t(y) * w * 4;
    for (uint32_t x = 0; x < w; ++x) {  // BGR(A) -> RGBA
      dst[4 * x + 0] = src[px * x + 2];
      dst[4 * x + 1] = src[px * x + 1];
      dst[4 * x + 2] = src[px * x + 0];
      dst[4 * x + 3] = px == 4 ? src[px * x + 3] : 255;
    }
  }
  return NVPRO_PYRAMID_SUCCESS;
}

}  // extern "C"
