// ref_dispatch.cpp -- TEST INFRASTRUCTURE ONLY.
// Compiles the reference dispatcher (nvpro_pyramid/nvpro_pyramid_dispatch.hpp)
// as host C++ against the recording declarations of ref_shim/vulkan, and
// exports the sequence of commands it records for a given image size.  Built
// into oracle/_ref/libref_dispatch.so by oracle/Makefile; its output is the
// golden dispatch schedule for tests/golden/dispatch_schedules.json.
#include <cstdint>
#include <cstring>
#include <vector>

#include "nvpro_pyramid/nvpro_pyramid_dispatch.hpp"

namespace {
// Each event: {kind, a, b, c}; kind 1 = bind(pipeline id), 2 = push
// constant(value), 3 = dispatch(x, y, z), 4 = barrier.
std::vector<uint32_t> g_events;
const VkPipeline kGeneral = reinterpret_cast<VkPipeline>(uintptr_t(0x1000));
const VkPipeline kFast = reinterpret_cast<VkPipeline>(uintptr_t(0x2000));

void push(uint32_t k, uint32_t a, uint32_t b, uint32_t c) {
  g_events.insert(g_events.end(), {k, a, b, c});
}

uint32_t nullDispatcher(VkCommandBuffer, VkPipelineLayout, uint32_t, VkPipeline, const NvproPyramidState& s) {
  return s.remainingLevels;
}
}  // namespace

void vkCmdBindPipeline(VkCommandBuffer, VkPipelineBindPoint, VkPipeline p) {
  push(1, p == kFast ? 1u : p == kGeneral ? 0u : 99u, 0, 0);
}
void vkCmdPushConstants(VkCommandBuffer, VkPipelineLayout, VkShaderStageFlags, uint32_t offset, uint32_t size,
                        const void* pValues) {
  uint32_t v = 0;
  std::memcpy(&v, pValues, size < 4 ? size : 4);
  push(2, v, offset, size);
}
void vkCmdDispatch(VkCommandBuffer, uint32_t x, uint32_t y, uint32_t z) { push(3, x, y, z); }
void vkCmdPipelineBarrier(VkCommandBuffer, VkPipelineStageFlags, VkPipelineStageFlags, VkDependencyFlags, uint32_t,
                          const VkMemoryBarrier*, uint32_t, const VkBufferMemoryBarrier*, uint32_t,
                          const VkImageMemoryBarrier*) {
  push(4, 0, 0, 0);
}

extern "C" {

// variant: 0 default <4,6>; 1 <2,5>; 2 <2,6>; 3 null fast dispatcher;
// 4 null general dispatcher (fast default).  hasFast = 0: no fast pipeline.
// Writes 4 words per event; returns the event count or -1 on overflow.
int ref_dispatch_events(uint32_t w, uint32_t h, uint32_t mipLevels, int hasFast, int variant, uint32_t* out,
                        int maxEvents) {
  g_events.clear();
  NvproPyramidPipelines p;
  p.generalPipeline = kGeneral;
  p.fastPipeline = hasFast ? kFast : VK_NULL_HANDLE;
  VkCommandBuffer cmd = reinterpret_cast<VkCommandBuffer>(uintptr_t(0x3000));
  nvpro_pyramid_dispatcher_t general = nvproPyramidDefaultGeneralDispatcher;
  nvpro_pyramid_dispatcher_t fast = nvproPyramidDefaultFastDispatcher;
  if (variant == 1) fast = nvproPyramidDefaultFastDispatcher<2, 5>;
  if (variant == 2) fast = nvproPyramidDefaultFastDispatcher<2, 6>;
  if (variant == 3) fast = nullDispatcher;
  if (variant == 4) general = nullDispatcher;
  nvproCmdPyramidDispatch(cmd, p, w, h, mipLevels, general, fast);
  const int n = (int)(g_events.size() / 4);
  if (n > maxEvents) return -1;
  std::memcpy(out, g_events.data(), g_events.size() * sizeof(uint32_t));
  return n;
}
}
