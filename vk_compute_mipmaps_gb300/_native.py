"""ctypes bindings of include/nvpro_pyramid_cuda.h (libnvpro_pyramid_cuda.so).

The library is built in-tree by vk_compute_mipmaps_gb300._build (or
__graft_entry__.build()).  Loading fails loudly if it is missing: there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_int, c_uint16, c_uint32, c_uint64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().with_name("libnvpro_pyramid_cuda.so")
MAX_LEVELS = 32
INPUT_LEVEL_SHIFT = 5

SUCCESS = 0
ERROR_INVALID_ARGUMENT = 1
ERROR_INVALID_STATE = 2
ERROR_DISPATCHER = 3
ERROR_UNSUPPORTED = 4
ERROR_CUDA = 5
ERROR_OUT_OF_MEMORY = 6
ERROR_TIMEOUT = 7
ERROR_IO = 8

PRESET_SRGBA8 = 1
PRESET_RGBA32F = 2
PRESET_RGBA16F = 3

CMD_RECORD_ONLY = 0x1
CMD_NO_FUSION = 0x2
CMD_PORTABLE_KERNELS = 0x4

CONFIG_SRGB_SHARED = 0x1
CONFIG_F16_SHARED = 0x2
CONFIG_NO_BILINEAR = 0x4


class NvproPyramidImage(ctypes.Structure):
    _fields_ = [
        ("width", c_uint32),
        ("height", c_uint32),
        ("levelCount", c_uint32),
        ("reserved", c_uint32),
        ("levels", c_void_p * MAX_LEVELS),
        ("rowPitchBytes", c_uint64 * MAX_LEVELS),
    ]


class NvproPyramidPipelines(ctypes.Structure):
    _fields_ = [
        ("generalPipeline", c_void_p),
        ("fastPipeline", c_void_p),
        ("layout", c_void_p),
        ("pushConstantOffset", c_uint32),
    ]


class NvproPyramidState(ctypes.Structure):
    _fields_ = [
        ("currentLevel", c_uint32),
        ("remainingLevels", c_uint32),
        ("currentX", c_uint32),
        ("currentY", c_uint32),
    ]


class NvproPyramidDispatchRecord(ctypes.Structure):
    _fields_ = [
        ("isFastPipeline", c_uint32),
        ("preset", c_uint32),
        ("pushConstant", c_uint32),
        ("groupCountX", c_uint32),
        ("groupCountY", c_uint32),
        ("groupCountZ", c_uint32),
        ("pipelineBound", c_uint32),
        ("barrierBefore", c_uint32),
        ("configBits", c_uint32),
        ("isBlit", c_uint32),
    ]


class NvproPyramidBatchInfo(ctypes.Structure):
    _fields_ = [
        ("imageCount", c_uint32),
        ("phaseCount", c_uint32),
        ("jobCount", c_uint32),
        ("stripBand", c_uint32),
        ("unitCount", c_uint64),
        ("autotuned", c_uint32),
        ("fromCache", c_uint32),
        ("graph", c_uint32),
        ("fastRegionRows", c_uint32),
        ("threadsPerCta", c_uint32),
        ("fromDisk", c_uint32),
    ]


BATCH_AUTOTUNE = 1
BATCH_GRAPH = 2
BATCH_RETUNE = 4

# nvpro_pyramid_dispatcher_t
DISPATCHER = ctypes.CFUNCTYPE(c_uint32, c_void_p, c_void_p, c_uint32, c_void_p, POINTER(NvproPyramidState))

# name -> (restype, argtypes); every function the header declares.
SIGNATURES = {
    "nvproPyramidResultString": (c_char_p, [c_int]),
    "nvproPyramidLastError": (c_char_p, []),
    "nvproPyramidCreatePipeline": (c_int, [c_int, c_uint32, POINTER(c_void_p)]),
    "nvproPyramidCreatePipelineEx": (c_int, [c_int, c_uint32, c_uint32, POINTER(c_void_p)]),
    # launcher as a function address (nvpro_pyramid_launcher_t, from a compiled functor set)
    "nvproPyramidCreateCustomPipeline": (c_int, [c_uint32, c_uint32, c_void_p, c_void_p, POINTER(c_void_p)]),
    "nvproPyramidDebugForceWaitTimeout": (c_int, [c_void_p, c_uint32]),
    "nvproPyramidSpeedOfLightProbe": (c_int, [c_void_p, POINTER(NvproPyramidImage), c_uint32]),
    "nvproPyramidPremultiplyAlpha": (c_int, [c_void_p, c_void_p, c_uint64, c_void_p, c_uint64, c_uint32, c_uint32]),
    "nvproPyramidWriteTga": (c_int, [c_char_p, c_void_p, c_uint32, c_uint32, c_uint64]),
    "nvproPyramidWriteLevelsTga": (c_int, [c_char_p, c_void_p, c_uint32, c_uint32, c_uint32]),
    "nvproPyramidReadTga": (c_int, [c_char_p, c_void_p, c_uint64, POINTER(c_uint32), POINTER(c_uint32)]),
    "nvproPyramidDestroyPipeline": (None, [c_void_p]),
    "nvproPyramidPresetTexelBytes": (c_uint32, [c_int]),
    "nvproPyramidFullLevelCount": (c_uint32, [c_uint32, c_uint32]),
    "nvproPyramidPackedLayout": (c_int, [c_uint32, c_uint32, c_uint32, c_uint32, POINTER(c_uint64)]),
    "nvproPyramidImageInitPacked": (c_int, [POINTER(NvproPyramidImage), c_void_p, c_uint32, c_uint32,
                                            c_uint32, c_uint32]),
    "nvproPyramidCreateCmd": (c_int, [c_uint32, POINTER(c_void_p)]),
    "nvproPyramidDestroyCmd": (None, [c_void_p]),
    "nvproPyramidBeginCmd": (c_int, [c_void_p, c_void_p]),
    "nvproPyramidEndCmd": (c_int, [c_void_p]),
    "nvproPyramidCmdBindImage": (c_int, [c_void_p, POINTER(NvproPyramidImage)]),
    "nvproPyramidCmdBindPipeline": (c_int, [c_void_p, c_void_p]),
    "nvproPyramidCmdPushConstants": (c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p]),
    "nvproPyramidCmdDispatch": (c_int, [c_void_p, c_uint32, c_uint32, c_uint32]),
    "nvproPyramidCmdPipelineBarrier": (c_int, [c_void_p]),
    "nvproPyramidCmdRecordCount": (c_uint32, [c_void_p]),
    "nvproPyramidCmdGetRecords": (c_int, [c_void_p, POINTER(NvproPyramidDispatchRecord), c_uint32]),
    "nvproPyramidCmdLaunchCount": (c_uint32, [c_void_p]),
    "nvproCmdPyramidDispatch": (c_int, [c_void_p, NvproPyramidPipelines, c_uint32, c_uint32, c_uint32]),
    "nvproCmdPyramidDispatchEx": (c_int, [c_void_p, NvproPyramidPipelines, c_uint32, c_uint32, c_uint32,
                                          DISPATCHER, DISPATCHER]),
    "nvproPyramidDefaultFastDispatcher": (c_uint32, [c_void_p, c_void_p, c_uint32, c_void_p,
                                                     POINTER(NvproPyramidState)]),
    "nvproPyramidFastDispatch": (c_uint32, [c_void_p, c_void_p, c_uint32, c_void_p, POINTER(NvproPyramidState),
                                            c_uint32, c_uint32]),
    "nvproPyramidCmdBlitLevel": (c_int, [c_void_p, c_uint32]),
    "nvproPyramidBlitGeneralDispatcher": (c_uint32, [c_void_p, c_void_p, c_uint32, c_void_p,
                                                     POINTER(NvproPyramidState)]),
    "nvproPyramidDefaultGeneralDispatcher": (c_uint32, [c_void_p, c_void_p, c_uint32, c_void_p,
                                                        POINTER(NvproPyramidState)]),
    "nvproPyramidCmdDeviceStatus": (c_int, [c_void_p]),
    "nvproPyramidDebugSrgbEncode": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint64]),
    "nvproPyramidDebugAlphaEncode": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint64]),
    "nvproPyramidCreateBatch": (c_int, [c_int, c_uint32, POINTER(c_void_p)]),
    "nvproPyramidDestroyBatch": (None, [c_void_p]),
    "nvproPyramidBatchBuild": (c_int, [c_void_p, c_void_p, POINTER(NvproPyramidImage), c_uint32, c_uint32]),
    "nvproPyramidBatchSetStripBand": (c_int, [c_void_p, c_uint32]),
    "nvproPyramidBatchSetTuning": (c_int, [c_void_p, c_uint32, c_uint32, c_uint32]),
    "nvproPyramidBatchLaunch": (c_int, [c_void_p, c_void_p]),
    "nvproPyramidBatchGetInfo": (c_int, [c_void_p, POINTER(NvproPyramidBatchInfo)]),
    "nvproPyramidBatchDeviceStatus": (c_int, [c_void_p]),
    "nvproPyramidAdjointWorkspaceBytes": (c_uint64, [c_uint32, c_uint32, c_uint32]),
    "nvproPyramidAdjoint": (c_int, [c_void_p, c_int, POINTER(NvproPyramidImage), c_void_p, c_uint64, c_uint32,
                                    c_void_p, c_uint64]),
    "nvproPyramidGenerateNoAlloc": (c_int, [c_void_p, c_int, POINTER(NvproPyramidImage), c_uint32]),
    "nvproPyramidNoAllocDeviceStatus": (c_int, [c_void_p]),
    "nvproPyramidDebugNoAllocForceWaitTimeout": (c_int, [c_void_p, c_uint32]),
    # image / stride arrays by address (the autograd helpers pass numpy buffers)
    "nvproPyramidGenerateStrided": (c_int, [c_void_p, c_void_p, NvproPyramidPipelines, c_void_p, c_void_p, c_uint32,
                                            c_uint32]),
    "nvproPyramidAdjointStrided": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_uint64, c_uint64,
                                           c_uint32, c_uint32, c_void_p, c_uint64]),
    "nvproPyramidGenerate": (c_int, [c_void_p, c_void_p, NvproPyramidPipelines, POINTER(NvproPyramidImage),
                                     c_uint32]),
}

_lib = None


class NativeLibraryError(RuntimeError):
    """The native library is missing or a call into it failed."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def load() -> ctypes.CDLL:
    """Load libnvpro_pyramid_cuda.so (once) and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH.name} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int, what: str = "") -> None:
    """Raise NativeLibraryError for a non-success NvproPyramidResult."""
    if code != SUCCESS:
        lib = load()
        name = lib.nvproPyramidResultString(code).decode()
        detail = lib.nvproPyramidLastError().decode()
        raise NativeLibraryError(code, f"{what}: {name} ({detail})" if what else f"{name} ({detail})")
