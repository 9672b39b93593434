// Declarations of the few Vulkan types and commands that
// nvpro_pyramid/nvpro_pyramid_dispatch.hpp uses, so that the reference
// dispatcher compiles as plain host C++.  The vkCmd* functions are defined by
// oracle/ref_dispatch.cpp, which records every call.  No graphics API is
// involved.  TEST INFRASTRUCTURE ONLY (oracle/_ref build).
#pragma once
#include <stdint.h>

typedef struct VkCommandBuffer_T* VkCommandBuffer;
typedef struct VkPipeline_T* VkPipeline;
typedef struct VkPipelineLayout_T* VkPipelineLayout;
#define VK_NULL_HANDLE nullptr

typedef uint32_t VkFlags;
typedef VkFlags VkAccessFlags;
typedef VkFlags VkPipelineStageFlags;
typedef VkFlags VkDependencyFlags;
typedef VkFlags VkShaderStageFlags;

typedef enum VkStructureType { VK_STRUCTURE_TYPE_MEMORY_BARRIER = 46 } VkStructureType;
typedef enum VkAccessFlagBits {
  VK_ACCESS_SHADER_READ_BIT  = 0x00000020,
  VK_ACCESS_SHADER_WRITE_BIT = 0x00000040
} VkAccessFlagBits;
typedef enum VkPipelineStageFlagBits { VK_PIPELINE_STAGE_COMPUTE_SHADER_BIT = 0x00000800 } VkPipelineStageFlagBits;
typedef enum VkPipelineBindPoint { VK_PIPELINE_BIND_POINT_COMPUTE = 1 } VkPipelineBindPoint;
typedef enum VkShaderStageFlagBits { VK_SHADER_STAGE_COMPUTE_BIT = 0x00000020 } VkShaderStageFlagBits;

typedef struct VkMemoryBarrier {
  VkStructureType sType;
  const void*     pNext;
  VkAccessFlags   srcAccessMask;
  VkAccessFlags   dstAccessMask;
} VkMemoryBarrier;
typedef struct VkBufferMemoryBarrier VkBufferMemoryBarrier;
typedef struct VkImageMemoryBarrier VkImageMemoryBarrier;

void vkCmdBindPipeline(VkCommandBuffer, VkPipelineBindPoint, VkPipeline);
void vkCmdPushConstants(VkCommandBuffer, VkPipelineLayout, VkShaderStageFlags, uint32_t offset,
                        uint32_t size, const void* pValues);
void vkCmdDispatch(VkCommandBuffer, uint32_t x, uint32_t y, uint32_t z);
void vkCmdPipelineBarrier(VkCommandBuffer, VkPipelineStageFlags, VkPipelineStageFlags, VkDependencyFlags,
                          uint32_t, const VkMemoryBarrier*, uint32_t, const VkBufferMemoryBarrier*, uint32_t,
                          const VkImageMemoryBarrier*);
