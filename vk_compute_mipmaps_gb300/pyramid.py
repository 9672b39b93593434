"""Python mirror of the nvpro_pyramid host interface over the C ABI.

Names follow nvpro_pyramid/nvpro_pyramid_dispatch.hpp: Pipelines is
NvproPyramidPipelines, Cmd is the command buffer that nvproCmdPyramidDispatch
records into, and cmd_pyramid_dispatch is nvproCmdPyramidDispatch itself.
MipChain is a convenience for torch users: a packed device allocation in the
layout of include/mipmap_storage.hpp:53-76 (levels contiguous, each [y][x]).
"""
from __future__ import annotations

import ctypes
import threading
from typing import Callable, Optional, Sequence

from . import _native as N

PRESET_BYTES = {N.PRESET_SRGBA8: 4, N.PRESET_RGBA32F: 16, N.PRESET_RGBA16F: 8}


def full_level_count(width: int, height: int) -> int:
    """floor(log2(max(w, h))) + 1 (nvpro_pyramid_dispatch.hpp:122-132)."""
    m = 0
    while width or height:
        width >>= 1
        height >>= 1
        m += 1
    return m


def level_sizes(width: int, height: int, levels: int = 0) -> list[tuple[int, int]]:
    levels = levels or full_level_count(width, height)
    return [(max(width >> k, 1), max(height >> k, 1)) for k in range(levels)]


def packed_offsets(width: int, height: int, levels: int, bytes_per_texel: int) -> list[int]:
    """Byte offset of each level in the packed layout, plus the total size."""
    offs, o = [], 0
    for w, h in level_sizes(width, height, levels):
        offs.append(o)
        o += w * h * bytes_per_texel
    return offs + [o]


class Pipelines:
    """NvproPyramidPipelines of one preset (nvpro_pyramid_dispatch.hpp:29-35)."""

    def __init__(self, preset: int = N.PRESET_SRGBA8, fast: bool = True):
        lib = N.load()
        self.preset = preset
        self._general = ctypes.c_void_p()
        self._fast = ctypes.c_void_p()
        N.check(lib.nvproPyramidCreatePipeline(preset, 0, ctypes.byref(self._general)), "create general pipeline")
        if fast:
            N.check(lib.nvproPyramidCreatePipeline(preset, 1, ctypes.byref(self._fast)), "create fast pipeline")

    @property
    def struct(self) -> N.NvproPyramidPipelines:
        return N.NvproPyramidPipelines(self._general.value, self._fast.value, None, 0)

    @property
    def general(self) -> Optional[int]:
        return self._general.value

    @property
    def fast(self) -> Optional[int]:
        return self._fast.value

    def close(self) -> None:
        lib = N.load()
        for h in (self._general, self._fast):
            if h.value:
                lib.nvproPyramidDestroyPipeline(h)
                h.value = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_image(levels: Sequence[int], width: int, height: int,
               pitches: Optional[Sequence[int]] = None) -> N.NvproPyramidImage:
    """NvproPyramidImage from per-level device addresses (and row pitches)."""
    img = N.NvproPyramidImage()
    img.width, img.height, img.levelCount = width, height, len(levels)
    for k, ptr in enumerate(levels):
        img.levels[k] = ptr
        img.rowPitchBytes[k] = pitches[k] if pitches else 0
    return img


class Cmd:
    """Command recorder bound to a CUDA stream (VkCommandBuffer analogue)."""

    def __init__(self, flags: int = 0):
        self._lib = N.load()
        self._h = ctypes.c_void_p()
        N.check(self._lib.nvproPyramidCreateCmd(flags, ctypes.byref(self._h)), "create command")
        self._keep: list = []

    @property
    def handle(self) -> int:
        return self._h.value

    def begin(self, stream: Optional[int] = None) -> "Cmd":
        """stream: a cudaStream_t as an int (e.g. torch.cuda.current_stream().cuda_stream)."""
        self._keep = []
        N.check(self._lib.nvproPyramidBeginCmd(self._h, stream), "begin")
        return self

    def bind_image(self, image: N.NvproPyramidImage) -> None:
        self._keep.append(image)
        N.check(self._lib.nvproPyramidCmdBindImage(self._h, ctypes.byref(image)), "bind image")

    def bind_pipeline(self, pipeline: int) -> None:
        N.check(self._lib.nvproPyramidCmdBindPipeline(self._h, pipeline), "bind pipeline")

    def push_constant(self, value: int) -> None:
        v = ctypes.c_uint32(value)
        N.check(self._lib.nvproPyramidCmdPushConstants(self._h, None, 0, 4, ctypes.byref(v)), "push constant")

    def dispatch(self, gx: int, gy: int = 1, gz: int = 1) -> None:
        N.check(self._lib.nvproPyramidCmdDispatch(self._h, gx, gy, gz), "dispatch")

    def barrier(self) -> None:
        N.check(self._lib.nvproPyramidCmdPipelineBarrier(self._h), "barrier")

    def end(self) -> None:
        N.check(self._lib.nvproPyramidEndCmd(self._h), "end")

    def records(self) -> list[dict]:
        n = self._lib.nvproPyramidCmdRecordCount(self._h)
        arr = (N.NvproPyramidDispatchRecord * max(n, 1))()
        N.check(self._lib.nvproPyramidCmdGetRecords(self._h, arr, n), "records")
        return [{f: getattr(arr[i], f) for f, _ in N.NvproPyramidDispatchRecord._fields_} for i in range(n)]

    @property
    def launch_count(self) -> int:
        return self._lib.nvproPyramidCmdLaunchCount(self._h)

    def close(self) -> None:
        if self._h.value:
            self._lib.nvproPyramidDestroyCmd(self._h)
            self._h.value = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


Dispatcher = Callable[[int, Optional[int], int, Optional[int], N.NvproPyramidState], int]


def wrap_dispatcher(fn: Dispatcher):
    """Turn fn(cmd, layout, push_constant_offset, pipeline_if_needed, state) into a C callback."""

    def trampoline(cmd, layout, pco, pipeline, state_ptr):
        return int(fn(cmd, layout, pco, pipeline, state_ptr.contents))

    return N.DISPATCHER(trampoline)


def cmd_pyramid_dispatch(cmd: Cmd, pipelines: Pipelines, width: int, height: int, mip_levels: int = 0,
                         general=None, fast=None) -> None:
    """nvproCmdPyramidDispatch (nvpro_pyramid_dispatch.hpp:54-59, :109-188).

    general / fast: optional dispatcher callbacks, either Python callables
    (see wrap_dispatcher) or ctypes function pointers of the library's own
    dispatchers; None selects the defaults.
    """
    lib = N.load()
    if general is None and fast is None:
        N.check(lib.nvproCmdPyramidDispatch(cmd.handle, pipelines.struct, width, height, mip_levels),
                "nvproCmdPyramidDispatch")
        return
    g = general if general is not None else N.DISPATCHER(("nvproPyramidDefaultGeneralDispatcher", lib))
    f = fast if fast is not None else N.DISPATCHER(("nvproPyramidDefaultFastDispatcher", lib))
    g = wrap_dispatcher(g) if callable(g) and not isinstance(g, ctypes._CFuncPtr) else g
    f = wrap_dispatcher(f) if callable(f) and not isinstance(f, ctypes._CFuncPtr) else f
    cmd._keep += [g, f]
    N.check(lib.nvproCmdPyramidDispatchEx(cmd.handle, pipelines.struct, width, height, mip_levels, g, f),
            "nvproCmdPyramidDispatchEx")


# ---------------------------------------------------------------------------
# torch convenience: packed mip chains on the GPU.

_DTYPES = {N.PRESET_SRGBA8: "uint8", N.PRESET_RGBA32F: "float32", N.PRESET_RGBA16F: "float16"}


class MipChain:
    """A packed mip chain in device memory: `storage` is a flat uint8 tensor."""

    def __init__(self, width: int, height: int, preset: int = N.PRESET_SRGBA8, levels: int = 0,
                 device="cuda", storage=None):
        import torch
        self.width, self.height, self.preset = width, height, preset
        self.levels = levels or full_level_count(width, height)
        self.bpp = PRESET_BYTES[preset]
        self.offsets = packed_offsets(width, height, self.levels, self.bpp)
        if storage is None:
            storage = torch.empty(self.offsets[-1], dtype=torch.uint8, device=device)
        assert storage.dtype == torch.uint8 and storage.numel() >= self.offsets[-1]
        self.storage = storage

    def level(self, k: int):
        """Level k as a [h, w, 4] tensor view of the preset's dtype."""
        import torch
        w, h = level_sizes(self.width, self.height, self.levels)[k]
        raw = self.storage[self.offsets[k]:self.offsets[k + 1]]
        return raw.view(getattr(torch, _DTYPES[self.preset])).view(h, w, 4)

    def image(self) -> N.NvproPyramidImage:
        base = self.storage.data_ptr()
        return make_image([base + o for o in self.offsets[:-1]], self.width, self.height)


_tls = threading.local()


def _defaults(preset: int, flags: int):
    key = (preset, flags)
    cache = getattr(_tls, "cache", None)
    if cache is None:
        cache = _tls.cache = {}
    if key not in cache:
        cache[key] = (Pipelines(preset), Cmd(flags))
    return cache[key]


def generate(chain: MipChain, stream: Optional[int] = None, mip_levels: int = 0, flags: int = 0,
             pipelines: Optional[Pipelines] = None, cmd: Optional[Cmd] = None) -> int:
    """Fill levels 1.. of `chain` from level 0 on `stream` (default: torch's
    current stream).  Returns the number of kernels launched."""
    import torch
    if stream is None:
        stream = torch.cuda.current_stream(chain.storage.device).cuda_stream
    p, c = _defaults(chain.preset, flags)
    pipelines = pipelines or p
    cmd = cmd or c
    img = chain.image()
    lib = N.load()
    N.check(lib.nvproPyramidGenerate(cmd.handle, stream, pipelines.struct, ctypes.byref(img),
                                     mip_levels or chain.levels), "nvproPyramidGenerate")
    return cmd.launch_count


class Batch:
    """Many sRGBA8 chains generated by one persistent launch
    (nvproPyramidCreateBatch / BatchBuild / BatchLaunch)."""

    def __init__(self, flags: int = 0, preset: int = N.PRESET_SRGBA8):
        self._lib = N.load()
        self._h = ctypes.c_void_p()
        N.check(self._lib.nvproPyramidCreateBatch(preset, flags, ctypes.byref(self._h)), "create batch")
        self._images = None

    def build(self, chains: Sequence["MipChain"], stream: Optional[int] = None, mip_levels: int = 0) -> None:
        import torch
        if stream is None:
            dev = chains[0].storage.device if chains else torch.device("cuda")
            stream = torch.cuda.current_stream(dev).cuda_stream
        arr = (N.NvproPyramidImage * max(len(chains), 1))()
        for i, c in enumerate(chains):
            arr[i] = c.image()
        self._images = arr  # the library copies them; kept for inspection
        N.check(self._lib.nvproPyramidBatchBuild(self._h, stream, arr, len(chains), mip_levels), "batch build")

    def set_strip_band(self, band: int) -> None:
        """Fix the general-pipeline unit size for the next build (0: default / autotuned)."""
        N.check(self._lib.nvproPyramidBatchSetStripBand(self._h, band), "batch strip band")

    def launch(self, stream: Optional[int] = None) -> None:
        import torch
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        N.check(self._lib.nvproPyramidBatchLaunch(self._h, stream), "batch launch")

    def info(self) -> dict:
        inf = N.NvproPyramidBatchInfo()
        N.check(self._lib.nvproPyramidBatchGetInfo(self._h, ctypes.byref(inf)), "batch info")
        return {name: getattr(inf, name) for name, _ in N.NvproPyramidBatchInfo._fields_ if name != "reserved"}

    def device_status(self) -> None:
        N.check(self._lib.nvproPyramidBatchDeviceStatus(self._h), "batch device status")

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if self._h.value:
            self._lib.nvproPyramidDestroyBatch(self._h)
            self._h.value = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pack_chains(sizes: Sequence[tuple], device="cuda", align: int = 256):
    """MipChains (sRGBA8) of the given (w, h) sizes in one device buffer, each
    starting on an `align`-byte boundary.  Returns (storage, chains)."""
    import torch
    offs, total = [], 0
    for w, h in sizes:
        offs.append(total)
        total += (packed_offsets(w, h, full_level_count(w, h), 4)[-1] + align - 1) // align * align
    storage = torch.empty(max(total, 1), dtype=torch.uint8, device=device)
    chains = []
    for (w, h), o in zip(sizes, offs):
        n = packed_offsets(w, h, full_level_count(w, h), 4)[-1]
        chains.append(MipChain(w, h, N.PRESET_SRGBA8, device=device, storage=storage[o:o + n]))
    return storage, chains
