"""GB300-native image-pyramid (mipmap) engine with the operator surface of
nvpro_pyramid (nvpro-samples/vk_compute_mipmaps).

The product is the native library libnvpro_pyramid_cuda.so (C ABI in
include/nvpro_pyramid_cuda.h, CUDA kernels for sm_103a).  This package loads
it through ctypes and adds torch conveniences; it has no CPU fallback.
"""
from . import _native
from ._native import (BATCH_AUTOTUNE, BATCH_GRAPH, CMD_NO_FUSION, CMD_PORTABLE_KERNELS, CMD_RECORD_ONLY,
                      CONFIG_F16_SHARED, CONFIG_NO_BILINEAR, CONFIG_SRGB_SHARED, PRESET_RGBA16F, PRESET_RGBA32F, PRESET_SRGBA8, NativeLibraryError, NvproPyramidImage,
                      NvproPyramidState)
from .pyramid import (Batch, Cmd, MipChain, Pipelines, blit_general_dispatcher, cmd_pyramid_dispatch, full_level_count, generate,
                      generate_from_host, level_sizes, make_image, pack_chains, packed_offsets, premultiply_alpha, read_tga,
                      wrap_dispatcher, write_levels_tga, write_tga)

__all__ = [
    "BATCH_AUTOTUNE", "BATCH_GRAPH", "Batch", "pack_chains", "generate_from_host", "CMD_NO_FUSION",
    "CMD_PORTABLE_KERNELS", "CMD_RECORD_ONLY", "CONFIG_F16_SHARED", "CONFIG_NO_BILINEAR", "CONFIG_SRGB_SHARED",
    "PRESET_RGBA16F", "PRESET_RGBA32F", "PRESET_SRGBA8", "NativeLibraryError", "NvproPyramidImage", "NvproPyramidState", "Cmd", "MipChain",
    "Pipelines", "blit_general_dispatcher", "cmd_pyramid_dispatch", "full_level_count", "generate", "level_sizes", "make_image",
    "packed_offsets", "premultiply_alpha", "wrap_dispatcher", "read_tga", "write_tga", "write_levels_tga",
]
